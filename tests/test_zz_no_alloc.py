"""The allocation-free solve entry point (mhfem_bicgstab_noalloc).

It serves callers whose device memory is owned by their own pool allocator
and who therefore cannot have this library call cudaMalloc / cudaFree: they
pass their own matrix, right-hand side and solution buffers, and the solver's
work vectors come from a fixed static device array.  The test builds the
caller-side buffers from the assembled system of the 128^2 heat-equation
workload (49,408 rows, below MHFEM_NOALLOC_MAX_ROWS), solves it through the
new entry point, and compares the solution with the one mhfem_solve (the
existing entry point) returns from the same warm start, on two consecutive
time steps.  It also checks that a system beyond the size limit is refused.
"""
import ctypes as ct

import numpy as np
import pytest

from helpers import rel_err
from mhfem import _lib as L
from mhfem import problems

pytestmark = pytest.mark.gpu

TOL_STATE = 1e-10


def _ell_from_csr(rowptr, cols, vals):
    """Unit-diagonal CSR -> off-diagonal ELL [width][rows] (padding = own row)."""
    rows = rowptr.size - 1
    lens = np.diff(rowptr) - 1
    W = int(lens.max())
    ecol = np.tile(np.arange(rows, dtype=np.int32), (W, 1))
    eval_ = np.zeros((W, rows))
    for r in range(rows):
        k = 0
        for q in range(rowptr[r], rowptr[r + 1]):
            if cols[q] == r:
                assert vals[q] == 1.0
                continue
            ecol[k, r] = cols[q]
            eval_[k, r] = vals[q]
            k += 1
    return W, ecol, eval_


def test_noalloc_solve_matches_mhfem_solve():
    import torch

    lib = L.load()
    p = problems.heat2d(N=128, steps=2)
    p.tol = 1e-12
    s = problems.make_solver(p)
    t = 0.0
    for _ in range(2):
        s.preIterate(t, p.dt)
        s.assembleLinearSystem(t, p.dt)
        rowptr, cols, vals, rhs = s.system()
        warm, _ = s.state()
        W, ecol, evals = _ell_from_csr(rowptr, cols, vals)
        d_cols = torch.from_numpy(np.ascontiguousarray(ecol)).cuda()
        d_vals = torch.from_numpy(np.ascontiguousarray(evals)).cuda()
        d_rhs = torch.from_numpy(rhs).cuda()
        d_x = torch.from_numpy(warm.copy()).cuda()
        torch.cuda.synchronize()
        it = ct.c_int32()
        res = ct.c_double()
        st = lib.mhfem_bicgstab_noalloc(d_cols.data_ptr(), d_vals.data_ptr(), W, rhs.size, d_rhs.data_ptr(),
                                        d_x.data_ptr(), p.tol, 20000, ct.byref(it), ct.byref(res), None)
        assert st == L.OK
        x_noalloc = d_x.cpu().numpy()
        ref = s.solveLinearSystem()
        zf, _ = s.state()
        assert res.value < p.tol and ref["residual"] < p.tol
        assert rel_err(x_noalloc, zf) < TOL_STATE
        s.postIterate(t, p.dt)
        t += p.dt
    s.close()


def test_noalloc_rejects_oversized_system():
    lib = L.load()
    it = ct.c_int32()
    res = ct.c_double()
    st = lib.mhfem_bicgstab_noalloc(None, None, 0, L.NOALLOC_MAX_ROWS + 1, None, None, 1e-10, 10,
                                    ct.byref(it), ct.byref(res), None)
    assert st == L.ERR_INVALID_ARGUMENT
