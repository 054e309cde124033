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


def _gravity_dy(p):
    """y(face centroid) - y(cell centroid) per local face e (opposite vertex
    e) of the triangles, [e][K]."""
    X = p.coords[p.cells]
    cen = X.mean(axis=1)
    out = []
    for e in range(3):
        others = [v for v in range(3) if v != e]
        out.append((X[:, others].mean(axis=1) - cen)[:, 1])
    return np.stack(out)


# packed index of b_ef in the triangle storage (MassMatrix.h:600-631)
_TRI_PACKED = [[0, 1, 3], [1, 2, 4], [3, 4, 5]]


def _run_gravity_model(place):
    """A model with a state-dependent D (updateNonLinearTerms) and a gravity
    term w_Ke = sum_f b_Kef (y_f - y_K) projected through b (its
    updateVectorCoefficients), on the GPU with the w update at `place`
    ("vector": the vector-coefficient hook, after this step's b; "pre": the
    pre-iterate hook, which sees the previous step's b), next to the oracle
    with the update where the reference makes it (Solver.hpp:641-652)."""
    import torch

    p = problems.heat2d(N=8, steps=4)
    p.tol = 1e-13
    C = p.cells.shape[0]
    D0 = np.linspace(0.5, 2.0, C)
    p.coeffs["D"] = D0.copy()
    p.coeffs["w"] = np.zeros(3 * C)
    dy = _gravity_dy(p)
    s = problems.make_solver(p)
    m = OracleModel.from_problem(p)

    def w_from_b(b, w):
        for e in range(3):
            i0, i1, i2 = _TRI_PACKED[e]
            w[e] = b[i0] * dy_t[0] + b[i1] * dy_t[1] + b[i2] * dy_t[2]

    def oracle_w(mm, t, tau):
        b = mm.b.reshape(9, C)
        w = mm.coeff_arrays["w"].reshape(3, C)
        for e in range(3):
            i0, i1, i2 = _TRI_PACKED[e]
            w[e] = b[i0] * dy[0] + b[i1] * dy[1] + b[i2] * dy[2]

    m.vector_hook = oracle_w
    D_dev = torch.as_tensor(s.coeff_device("D"), device="cuda")
    W_dev = torch.as_tensor(s.coeff_device("w"), device="cuda").view(3, C)
    B_dev = torch.as_tensor(s.array_device("b"), device="cuda").view(9, C)
    Z_dev = torch.as_tensor(s.array_device("Z_iK"), device="cuda")
    D0_dev = torch.tensor(D0, device="cuda")
    dy_t = torch.tensor(dy, device="cuda")

    def pre(t, tau, stream):
        with torch.cuda.stream(torch.cuda.ExternalStream(stream)):
            torch.mul(D0_dev, 1.0 + Z_dev * Z_dev, out=D_dev)
            if place == "pre":
                w_from_b(B_dev, W_dev)

    def vec(t, tau, stream):
        with torch.cuda.stream(torch.cuda.ExternalStream(stream)):
            w_from_b(B_dev, W_dev)

    s.set_hook(L.HOOK_PRE_ITERATE, pre)
    if place == "vector":
        s.set_hook(L.HOOK_VECTOR_COEFFICIENTS, vec)
    errs = []
    t = 0.0
    for _ in range(p.steps):
        m.coeff_arrays["D"][:] = D0 * (1.0 + m.Z_iK ** 2)
        s.step(t, p.dt)
        m.step(t, p.dt, 1e-14)
        zf, zk = s.state()
        errs.append((rel_err(zf, m.Z_iF), rel_err(zk, m.Z_iK)))
        t += p.dt
    w_gpu = W_dev.cpu().numpy().ravel()
    s.close()
    return errs, w_gpu, m.coeff_arrays["w"].copy()


def test_vector_coefficient_hook_sees_this_steps_b():
    """The vector-coefficient hook runs after the b update of the same step:
    a b-dependent w matches the oracle, which updates w between its b update
    and upwinding, at 1e-10 after every step.  The same update from the
    pre-iterate hook reads the previous step's b and misses by far more."""
    errs, w_gpu, w_orc = _run_gravity_model("vector")
    assert np.abs(w_orc).max() > 0
    assert rel_err(w_gpu, w_orc) < 1e-12
    for step, (ef, ek) in enumerate(errs):
        assert ef < 1e-10 and ek < 1e-10, f"step {step}: {ef:.2e} {ek:.2e}"
    lagged, _, _ = _run_gravity_model("pre")
    assert max(lagged[-1]) > 1e-6


def test_time_dependent_boundary_mobility_matches_oracle():
    """getBoundaryMobility as a function of (E, t) (Solver.hpp:690-700): a model
    rewrites m_bnd from the vector-coefficient hook every step, and the
    mobility upwinding of the same step takes it on the inflow faces (x = 0,
    Dirichlet 1 into a domain at 0).  The oracle evaluates the same function
    at the same point; each step starts from the GPU's velocities (the upwind
    choice is a sign test that can flip at rounding level, as in
    test_step_parity)."""
    import torch

    p = problems.diffusion3d(N=4, steps=4)
    p.tol = 1e-13
    rng = np.random.default_rng(5)
    C = p.C
    base_bc = p.bc_fn

    def bc_inflow(fv, fc):
        tags, vals, dirichlet = base_bc(fv, fc)
        from mhfem import meshgen
        x = meshgen.face_centroids(p.coords, fv)[:, 0]
        dirichlet = np.where((fc[:, 1] < 0) & (np.abs(x) < 1e-12), 1.0, 0.0)
        return tags, vals, dirichlet

    p.bc_fn = bc_inflow
    p.config.mobility_upwind = True
    p.coeffs["m"] = rng.uniform(0.5, 2.0, C)
    s = problems.make_solver(p)
    F = s.F
    fv, _, _ = s.topology()
    from mhfem import meshgen
    y = meshgen.face_centroids(p.coords, fv)[:, 1]
    p.coeffs["m_bnd"] = np.ones(F)
    s.set_coeff("m_bnd", p.coeffs["m_bnd"])
    m = OracleModel.from_problem(p)

    def g(t):
        return 1.0 + 0.5 * np.sin(2 * np.pi * t / (4 * p.dt))

    y_dev = torch.tensor(y, device="cuda")
    mb_dev = torch.as_tensor(s.coeff_device("m_bnd"), device="cuda")
    assert mb_dev.numel() == F

    def vec(t, tau, stream):
        with torch.cuda.stream(torch.cuda.ExternalStream(stream)):
            torch.mul(1.0 + y_dev, g(t), out=mb_dev)

    def oracle_vec(mm, t, tau):
        mm.coeff_arrays["m_bnd"][:] = (1.0 + y) * g(t)

    s.set_hook(L.HOOK_VECTOR_COEFFICIENTS, vec)
    m.vector_hook = oracle_vec
    nf = 4
    t = 0.0
    used_inflow = False
    for step in range(p.steps):
        if step > 0:
            m.v_iKe[:] = s.array("v_iKe", nf * C)
        s.step(t, p.dt)
        m.step(t, p.dt, 1e-14)
        zf, zk = s.state()
        assert rel_err(zf, m.Z_iF) < 1e-10, f"step {step}"
        assert rel_err(zk, m.Z_iK) < 1e-10, f"step {step}"
        mu = s.array("m_upw", F)
        assert rel_err(mu, m.m_upw) < 1e-12
        bnd_in = np.isclose(mu, (1.0 + y) * g(t), rtol=0, atol=1e-15) & (np.abs(mu - 1.0) > 1e-3)
        used_inflow = used_inflow or bool(bnd_in.any())
        t += p.dt
    assert used_inflow  # some faces took the model's boundary mobility
    s.close()
