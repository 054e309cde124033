"""The bounded grid barrier of the small-system FP64 BiCGStab (one
cooperative launch per solve on systems of at most 2^18 rows).

Every wait of that barrier gives up after a poll limit, sets a failure flag
the host reads, and returns, so a CTA that never arrives ends the launch
with an error status instead of a hang.  The check launches the barrier
with every CTA arriving (all pass), then with one CTA that never arrives
and a short limit (the others give up and set the flag), and finally runs a
solve on the same device to show the context stayed usable.  Nothing here
faults or hangs a GPU: the waits that run out are bounded by design.
"""
import ctypes as ct

import numpy as np
import pytest

from mhfem import _lib as L
from mhfem import problems

pytestmark = pytest.mark.gpu


def _check(lib, ctas, skip, polls):
    passed, gave_up, flag = ct.c_int32(), ct.c_int32(), ct.c_int32()
    st = lib.mhfem_check_grid_barrier(0, ctas, skip, polls, ct.byref(passed), ct.byref(gave_up), ct.byref(flag))
    return st, passed.value, gave_up.value, flag.value


def test_grid_barrier_passes_when_every_cta_arrives():
    lib = L.load()
    st, passed, gave_up, flag = _check(lib, 8, -1, 1 << 22)
    assert st == L.OK
    assert (passed, gave_up, flag) == (8, 0, 0)


def test_grid_barrier_wait_runs_out_and_reports():
    lib = L.load()
    st, passed, gave_up, flag = _check(lib, 8, 3, 4096)
    assert st == L.OK
    assert passed == 0 and gave_up == 7 and flag == 1
    # the context is intact: a small-system solve on the same device converges
    p = problems.heat2d(N=32, steps=2)
    s = problems.make_solver(p)
    t = 0.0
    for _ in range(p.steps):
        out = s.step(t, p.dt)
        assert out["residual"] < p.tol
        t += p.dt
    zf, _ = s.state()
    assert np.isfinite(zf).all()
    s.close()


def test_grid_barrier_rejects_bad_arguments():
    lib = L.load()
    st, *_ = _check(lib, 0, -1, 16)
    assert st == L.ERR_INVALID_ARGUMENT
    st, *_ = _check(lib, 8, -1, 0)
    assert st == L.ERR_INVALID_ARGUMENT
