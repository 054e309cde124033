"""Model hooks through the C ABI (needs a GB300): a custom nonlinear model
updates its coefficients on the device in place each step, as a reference
model's updateNonLinearTerms does (Solver.hpp:616-625)."""
import numpy as np
import pytest

from helpers import rel_err
from mhfem import _lib as L
from mhfem import problems
from oracle.oracle import OracleModel

pytestmark = pytest.mark.gpu


def test_nonlinear_diffusion_hook_matches_oracle():
    """D_K = D0_K (1 + Z_K^2), recomputed before every step from the current
    cell values by a torch kernel on the library's stream that writes the
    library's own D array; the oracle applies the same update on the host."""
    import torch

    p = problems.heat2d(N=8, steps=4)
    p.tol = 1e-13
    C = p.cells.shape[0]
    D0 = np.linspace(0.5, 2.0, C)
    p.coeffs["D"] = D0.copy()
    s = problems.make_solver(p)
    m = OracleModel.from_problem(p)
    D_dev = torch.as_tensor(s.coeff_device("D"), device="cuda")
    Z_dev = torch.as_tensor(s.array_device("Z_iK"), device="cuda")
    assert D_dev.numel() == C and Z_dev.numel() == C
    D0_dev = torch.tensor(D0, device="cuda")
    calls = {"pre": 0, "post": 0}

    def pre(t, tau, stream):
        calls["pre"] += 1
        with torch.cuda.stream(torch.cuda.ExternalStream(stream)):
            torch.mul(D0_dev, 1.0 + Z_dev * Z_dev, out=D_dev)

    def post(t, tau, stream):
        calls["post"] += 1

    s.set_hook(L.HOOK_PRE_ITERATE, pre)
    s.set_hook(L.HOOK_POST_ITERATE, post)
    t = 0.0
    for _ in range(p.steps):
        m.coeff_arrays["D"][:] = D0 * (1.0 + m.Z_iK ** 2)
        s.step(t, p.dt)
        m.step(t, p.dt, 1e-14)
        t += p.dt
    zf, zk = s.state()
    assert calls == {"pre": p.steps, "post": p.steps}
    assert rel_err(zf, m.Z_iF) < 1e-10
    assert rel_err(zk, m.Z_iK) < 1e-10
    # the coefficient really changed: the run differs from the linear model
    q = problems.heat2d(N=8, steps=4)
    q.tol = 1e-13
    q.coeffs["D"] = D0.copy()
    lin = problems.make_solver(q)
    t = 0.0
    for _ in range(q.steps):
        lin.step(t, q.dt)
        t += q.dt
    assert rel_err(lin.state()[1], zk) > 1e-6
    s.set_hook(L.HOOK_PRE_ITERATE, None)
    s.close()
    lin.close()


def test_set_coeff_from_device_memory():
    """mhfem_set_coeff takes a device pointer as well as a host one."""
    import torch

    p = problems.diffusion3d(N=4, steps=1)
    p.tol = 1e-13
    D = np.asarray(p.coeffs["D"], np.float64)
    a = problems.make_solver(p)
    b = problems.make_solver(p)
    Dt = torch.tensor(D * 1.7, device="cuda")
    b._ck(b.lib.mhfem_set_coeff(b._h, L.COEF_D, ctypes_ptr(Dt), Dt.numel()))
    a.set_coeff("D", D * 1.7)
    a.step(0.0, p.dt)
    b.step(0.0, p.dt)
    assert np.array_equal(a.state()[0], b.state()[0])
    a.close()
    b.close()


def ctypes_ptr(t):
    import ctypes as ct

    return ct.cast(ct.c_void_p(t.data_ptr()), ct.POINTER(ct.c_double))
