"""The allocation-free solve entry point (mhfem_bicgstab_noalloc).

It serves callers whose device memory is owned by their own pool allocator
and who therefore cannot have this library call cudaMalloc / cudaFree: they
pass their own matrix, right-hand side and solution buffers, and the solver's
work vectors come from a fixed static device array.  The tests build the
caller-side buffers from the assembled systems of the 128^2 heat-equation
workload (49,408 rows) and of a 7^2 grid (161 rows, an odd count), solve them
through the new entry point, and compare the solutions with the ones
mhfem_solve (the existing entry point) returns from the same warm start, on
two consecutive time steps (both run the persistent small-system solve at
these sizes).  They also check that a repeated call leaves the
device's free memory unchanged, that a system beyond the size limit or with
a column index outside the system is refused, and that the wall-clock limit
ends a solve that cannot converge with MHFEM_ERR_TIMEOUT.
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


def _device_system(s):
    """The solver's current system as caller-owned device buffers."""
    import torch

    rowptr, cols, vals, rhs = s.system()
    warm, _ = s.state()
    W, ecol, evals = _ell_from_csr(rowptr, cols, vals)
    d = {"W": W, "rows": rhs.size,
         "cols": torch.from_numpy(np.ascontiguousarray(ecol)).cuda(),
         "vals": torch.from_numpy(np.ascontiguousarray(evals)).cuda(),
         "rhs": torch.from_numpy(rhs).cuda(), "x": torch.from_numpy(warm.copy()).cuda()}
    torch.cuda.synchronize()
    return d


def _call(lib, d, tol, max_iter=20000, timeout_s=0.0):
    it = ct.c_int32()
    res = ct.c_double()
    st = lib.mhfem_bicgstab_noalloc(d["cols"].data_ptr(), d["vals"].data_ptr(), d["W"], d["rows"],
                                    d["rhs"].data_ptr(), d["x"].data_ptr(), tol, max_iter, timeout_s,
                                    ct.byref(it), ct.byref(res), None)
    return st, it.value, res.value


@pytest.mark.parametrize("N", [128, 7])
def test_noalloc_solve_matches_mhfem_solve(N):
    """Two consecutive steps; N = 7 gives 161 rows, an odd count."""
    lib = L.load()
    p = problems.heat2d(N=N, steps=2)
    p.tol = 1e-12
    s = problems.make_solver(p)
    t = 0.0
    for _ in range(2):
        s.preIterate(t, p.dt)
        s.assembleLinearSystem(t, p.dt)
        d = _device_system(s)
        if N == 7:
            assert d["rows"] % 2 == 1
        st, _, res = _call(lib, d, p.tol)
        assert st == L.OK
        x_noalloc = d["x"].cpu().numpy()
        ref = s.solveLinearSystem()
        zf, _ = s.state()
        assert res < p.tol and ref["residual"] < p.tol
        assert rel_err(x_noalloc, zf) < TOL_STATE
        s.postIterate(t, p.dt)
        t += p.dt
    s.close()


def test_noalloc_leaves_device_memory_unchanged():
    """After a warm-up call (which commits the static array on the device), a
    further call changes the device's free memory by nothing."""
    import torch

    lib = L.load()
    p = problems.heat2d(N=64, steps=1)
    p.tol = 1e-12
    s = problems.make_solver(p)
    s.preIterate(0.0, p.dt)
    s.assembleLinearSystem(0.0, p.dt)
    d = _device_system(s)
    x0 = d["x"].clone()
    torch.cuda.synchronize()
    st, _, _ = _call(lib, d, p.tol)
    assert st == L.OK
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    d["x"].copy_(x0)
    torch.cuda.synchronize()
    st, _, _ = _call(lib, d, p.tol)
    assert st == L.OK
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0
    s.close()


def test_noalloc_rejects_oversized_system():
    lib = L.load()
    it = ct.c_int32()
    res = ct.c_double()
    st = lib.mhfem_bicgstab_noalloc(None, None, 0, L.NOALLOC_MAX_ROWS + 1, None, None, 1e-10, 10, 0.0,
                                    ct.byref(it), ct.byref(res), None)
    assert st == L.ERR_INVALID_ARGUMENT


def test_noalloc_rejects_column_outside_the_system():
    """One column index equal to the row count: the check pass refuses the
    system before any SpMV reads x at that index."""
    lib = L.load()
    p = problems.heat2d(N=16, steps=1)
    s = problems.make_solver(p)
    s.preIterate(0.0, p.dt)
    s.assembleLinearSystem(0.0, p.dt)
    d = _device_system(s)
    x0 = d["x"].clone()
    d["cols"][1, d["rows"] // 2] = d["rows"]
    st, _, _ = _call(lib, d, 1e-10)
    assert st == L.ERR_INVALID_ARGUMENT
    assert bool((d["x"] == x0).all())  # nothing ran
    d["cols"][1, d["rows"] // 2] = -1
    st, _, _ = _call(lib, d, 1e-10)
    assert st == L.ERR_INVALID_ARGUMENT
    s.close()


def test_noalloc_wall_clock_limit():
    """A tolerance no solve reaches and an iteration cap it never hits: the
    host-side limit ends the call with MHFEM_ERR_TIMEOUT, and the next call on
    the shared array solves normally."""
    lib = L.load()
    p = problems.heat2d(N=32, steps=1)
    s = problems.make_solver(p)
    s.preIterate(0.0, p.dt)
    s.assembleLinearSystem(0.0, p.dt)
    d = _device_system(s)
    x0 = d["x"].clone()
    st, it, _ = _call(lib, d, 1e-300, max_iter=1 << 30, timeout_s=1e-6)
    assert st == L.ERR_TIMEOUT
    assert 0 <= it < 1 << 30
    d["x"].copy_(x0)
    st, _, res = _call(lib, d, 1e-12)
    assert st == L.OK and res < 1e-12
    s.close()
