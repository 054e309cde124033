"""GPU path vs the CPU oracle, through the C ABI (needs a GB300).

Bars: topology, face numbering and the CSR pattern bit-exact; the local
quantities and the assembled values within 1e-12 relative; face traces and
cell averages within 1e-10 relative after each time step (both solves run
to a relative residual of 1e-13 so the comparison measures the path, not the
solver tolerance).
"""
import copy
import dataclasses

import numpy as np
import pytest

from helpers import diffusion3d_n2, golden_case, golden_names, rel_err, small_cases, variant
from mhfem import _lib as L
from mhfem import problems
from oracle.oracle import OracleModel

pytestmark = pytest.mark.gpu

CASES = small_cases()
TOL_LOCAL = 1e-12
TOL_STATE = 1e-10


def _pair(p, check_every=4):
    p.tol = 1e-13
    s = problems.make_solver(p, check_every=check_every)
    m = OracleModel.from_problem(p)
    return s, m


@pytest.mark.parametrize("name", sorted(CASES))
def test_topology_bit_exact(name):
    p = CASES[name]
    s, m = _pair(p)
    fv, fc, cf = s.topology()
    assert np.array_equal(fv, m.face_verts)
    assert np.array_equal(fc, m.face_cells)
    assert np.array_equal(cf, m.cell_faces)
    s.close()


@pytest.mark.parametrize("name", sorted(CASES))
def test_step_parity(name):
    p = CASES[name]
    s, m = _pair(p)
    n, C = p.n, p.C
    nf = p.config.faces_per_cell
    S = m.S
    t = 0.0
    for step in range(p.steps):
        if p.config.mobility_upwind and step > 0:
            # Mobility upwinding branches on the sign of v_K1 - v_K2 (Solver.hpp:
            # 711-720); where that difference is at rounding level the two
            # implementations may legitimately pick different cells.  Step-level
            # parity therefore starts each step from the GPU's velocities (which
            # were compared above at 1e-9).
            m.v_iKe[:] = s.array("v_iKe", n * nf * C)
        s.preIterate(t, p.dt)
        s.assembleLinearSystem(t, p.dt)
        m.pre_iterate(t, p.dt)
        m.assemble(t, p.dt)
        assert rel_err(s.array("b", n * n * S * C), m.b) < TOL_LOCAL
        assert rel_err(s.array("R_ijKe", n * n * nf * C), m.R_ijKe) < TOL_LOCAL
        assert rel_err(s.array("R_iK", n * C), m.R_iK) < TOL_LOCAL
        rowptr, cols, vals, rhs = s.system()
        assert np.array_equal(rowptr, m.rowptr), "CSR row pointers differ"
        assert np.array_equal(cols, m.cols), "CSR column indices differ"
        assert rel_err(vals, m.vals) < TOL_LOCAL
        assert rel_err(rhs, m.rhs) < TOL_LOCAL
        st = s.solveLinearSystem()
        m.solve(1e-13)
        s.postIterate(t, p.dt)
        m.post_iterate(t, p.dt)
        zf, zk = s.state()
        assert rel_err(zf, m.Z_iF) < TOL_STATE, f"step {step}: Z_iF"
        assert rel_err(zk, m.Z_iK) < TOL_STATE, f"step {step}: Z_iK"
        if p.config.mobility_upwind:
            assert rel_err(s.array("v_iKe", n * nf * C), m.v_iKe) < 1e-9
            assert rel_err(s.array("m_upw", n * p_faces(s)), m.m_upw) < 1e-12
        assert st["residual"] < 1e-13
        t += p.dt
    s.close()


def p_faces(s):
    return s.F


def _form_step_parity(name, form, **setup):
    """Every step of the case in the given form against the FP64 oracle at
    the FP64 bar, both solved to 1e-13 (the mobility-upwind cases start each
    step from the GPU's velocities, as in test_step_parity)."""
    p = variant(CASES[name], form=form)
    s, m = _pair(p)
    s.setup(tol=1e-13, max_iter=20000, check_every=4, **setup)
    n, C = p.n, p.C
    nf = p.config.faces_per_cell
    t = 0.0
    for step in range(p.steps):
        if p.config.mobility_upwind and step > 0:
            m.v_iKe[:] = s.array("v_iKe", n * nf * C)
        st = s.step(t, p.dt)
        m.step(t, p.dt, 1e-13)
        zf, zk = s.state()
        assert st["residual"] < 1e-13
        assert rel_err(zf, m.Z_iF) < TOL_STATE, f"step {step}: Z_iF"
        assert rel_err(zk, m.Z_iK) < TOL_STATE, f"step {step}: Z_iK"
        t += p.dt
    s.close()


@pytest.mark.parametrize("name", sorted(CASES))
def test_mixed_step_parity(name):
    """The mixed form (FP32 inner BiCGStab, FP64 iterative refinement) on
    every model case, refined to 1e-13: its FP64 outer residuals take it to
    FP64 accuracy, so it meets the FP64 form's 1e-10 bar against the oracle
    after every step -- n = 1 to 3, lumping, the advection schemes, mobility
    upwinding, box cells and the dummy-equation rows, through the FP32
    kernels of every ELL width."""
    _form_step_parity(name, L.FORM_MIXED, max_sweeps=60)


LEARNED_CASES = [n for n in sorted(CASES) if CASES[n].n == 1 and CASES[n].config.cell == L.CELL_SIMPLEX]


@pytest.mark.parametrize("name", LEARNED_CASES)
def test_learned_step_parity(name):
    """The learned form (one equation, simplex cells) on the model cases:
    its initial guess only changes where the FP64 solve starts, so every
    step meets the FP64 bar against the oracle."""
    _form_step_parity(name, L.FORM_LEARNED)


@pytest.mark.parametrize("name", golden_names())
def test_gpu_matches_golden(name):
    """The GPU path against the committed fixtures (tests/golden): inputs and
    expected outputs both read from the file, at the bars above."""
    p, d = golden_case(name)
    s = problems.make_solver(p, check_every=4)
    fv, fc, cf = s.topology()
    assert np.array_equal(fv, d["face_verts"])
    assert np.array_equal(fc, d["face_cells"])
    assert np.array_equal(cf, d["cell_faces"])
    n, C = p.n, p.C
    nf = p.config.faces_per_cell
    t = 0.0
    for step in range(p.steps):
        s.preIterate(t, p.dt)
        s.assembleLinearSystem(t, p.dt)
        if step == 0:
            assert rel_err(s.array("b", d["b0"].size), d["b0"]) < TOL_LOCAL
            assert rel_err(s.array("R_ijKe", n * n * nf * C), d["R_ijKe0"]) < TOL_LOCAL
            assert rel_err(s.array("R_iK", n * C), d["R_iK0"]) < TOL_LOCAL
            rowptr, cols, vals, rhs = s.system()
            assert np.array_equal(rowptr, d["rowptr"]) and np.array_equal(cols, d["cols"])
            assert rel_err(vals, d["vals0"]) < TOL_LOCAL
            assert rel_err(rhs, d["rhs0"]) < TOL_LOCAL
        s.solveLinearSystem()
        s.postIterate(t, p.dt)
        zf, zk = s.state()
        assert rel_err(zf, d["Z_iF"][step]) < TOL_STATE, f"step {step}: Z_iF"
        assert rel_err(zk, d["Z_iK"][step]) < TOL_STATE, f"step {step}: Z_iK"
        t += p.dt
    s.close()


def test_heat2d_full_size():
    """The 128^2 triangle heat-equation workload, 3 steps at tol 1e-12."""
    p = problems.heat2d(N=128, steps=3)
    s, m = _pair(p)
    assert s.F == 49408 and s.C == 32768
    t = 0.0
    for _ in range(p.steps):
        s.step(t, p.dt)
        m.step(t, p.dt, 1e-13)
        t += p.dt
    zf, zk = s.state()
    assert rel_err(zf, m.Z_iF) < TOL_STATE
    assert rel_err(zk, m.Z_iK) < TOL_STATE
    rowptr, cols, _, _ = s.system()
    assert np.array_equal(rowptr, m.rowptr) and np.array_equal(cols, m.cols)
    s.close()


def test_diffusion3d_full_size():
    """The 64^3 tetrahedral heterogeneous-diffusion workload: 2 steps."""
    p = problems.diffusion3d(N=64, steps=2)
    s, m = _pair(p, check_every=8)
    assert s.F == 3170304 and s.C == 1572864
    t = 0.0
    for _ in range(p.steps):
        s.step(t, p.dt)
        m.step(t, p.dt, 1e-13)
        t += p.dt
    zf, zk = s.state()
    assert rel_err(zf, m.Z_iF) < TOL_STATE
    assert rel_err(zk, m.Z_iK) < TOL_STATE
    rowptr, cols, _, _ = s.system()
    assert np.array_equal(rowptr, m.rowptr) and np.array_equal(cols, m.cols)
    s.close()


def test_adr2d_full_size():
    """The 512^2 two-component advection-diffusion-reaction workload (n = 2,
    mass lumping, explicit upwind, inflow / outflow / wall boundaries): 2
    steps against the oracle."""
    p = problems.adr2d(N=512, steps=2)
    s, m = _pair(p, check_every=8)
    assert s.C == 524288 and s.F == 787456
    t = 0.0
    for _ in range(p.steps):
        s.step(t, p.dt)
        m.step(t, p.dt, 1e-13)
        t += p.dt
    zf, zk = s.state()
    assert rel_err(zf, m.Z_iF) < TOL_STATE
    assert rel_err(zk, m.Z_iK) < TOL_STATE
    rowptr, cols, _, _ = s.system()
    assert np.array_equal(rowptr, m.rowptr) and np.array_equal(cols, m.cols)
    s.close()


def test_diffusion3d_n2_large():
    """Two components on the 24^3 tetrahedral mesh (338,688 rows, ELL width
    13, above the small-system size: the five-kernel FP64 iteration at that
    width): 2 steps against the oracle."""
    p = diffusion3d_n2(24)
    s, m = _pair(p, check_every=8)
    assert s.F * 2 > 1 << 18
    t = 0.0
    for _ in range(p.steps):
        s.step(t, p.dt)
        m.step(t, p.dt, 1e-13)
        t += p.dt
    zf, zk = s.state()
    assert rel_err(zf, m.Z_iF) < TOL_STATE
    assert rel_err(zk, m.Z_iK) < TOL_STATE
    s.close()


def test_heat2d_above_small_system_size():
    """The heat equation on a 300^2 triangle mesh (270,600 rows, ELL width
    4, just above the persistent small-system size): the five-kernel FP64
    iteration at width 4, 2 steps against the oracle."""
    p = problems.heat2d(N=300, steps=2)
    s, m = _pair(p, check_every=8)
    assert s.F > 1 << 18
    t = 0.0
    for _ in range(p.steps):
        s.step(t, p.dt)
        m.step(t, p.dt, 1e-13)
        t += p.dt
    zf, zk = s.state()
    assert rel_err(zf, m.Z_iF) < TOL_STATE
    assert rel_err(zk, m.Z_iK) < TOL_STATE
    s.close()


def test_box_full_size():
    """Box cells at full size: 128^2 graded rectangles (3 steps) and 64^3
    graded cuboids (2 steps) against the oracle; the pattern bit-exact."""
    for p in (problems.heat2d_rect(N=128, steps=3), problems.diffusion3d_box(N=64, steps=2)):
        s, m = _pair(p, check_every=8)
        t = 0.0
        for _ in range(p.steps):
            s.step(t, p.dt)
            m.step(t, p.dt, 1e-13)
            t += p.dt
        zf, zk = s.state()
        assert rel_err(zf, m.Z_iF) < TOL_STATE, p.name
        assert rel_err(zk, m.Z_iK) < TOL_STATE, p.name
        rowptr, cols, _, _ = s.system()
        assert np.array_equal(rowptr, m.rowptr) and np.array_equal(cols, m.cols)
        s.close()


def test_mixed_box():
    """Mixed precision on 32^3 cuboids: error against the FP64 oracle."""
    p = problems.diffusion3d_box(N=32, steps=3, form=L.FORM_MIXED)
    s = problems.make_solver(p)
    m = OracleModel.from_problem(p)
    t = 0.0
    for _ in range(p.steps):
        st = s.step(t, p.dt)
        m.step(t, p.dt, 1e-13)
        assert st["sweeps"] >= 1 and st["residual"] < p.tol
        t += p.dt
    zf, zk = s.state()
    assert rel_err(zf, m.Z_iF) < 1e-8
    assert rel_err(zk, m.Z_iK) < 1e-8
    s.close()


def test_mixed_128_cube():
    """Mixed precision on the 128^3 cube (12,582,912 tetrahedra, 25,264,128
    faces) over 2 steps at tol 1e-12: face traces and cell values within 1e-8
    of the GPU FP64 form, the final FP64 residual below the tolerance in
    every step (one step of both forms against the oracle:
    test_128_cube_against_oracle)."""
    p = problems.diffusion3d(N=128, steps=2, form=L.FORM_MIXED)
    p.tol = 1e-12  # at 1e-10 the two forms already differ by ~1.5e-8 through the tolerance alone
    sm = problems.make_solver(p, check_every=8)
    pf = copy.copy(p)
    pf.config = dataclasses.replace(p.config, form=L.FORM_FP64)
    sf = problems.make_solver(pf, check_every=8)
    assert sm.F == 25264128 and sm.C == 12582912
    t = 0.0
    for _ in range(p.steps):
        a = sm.step(t, p.dt)
        b = sf.step(t, p.dt)
        assert a["residual"] < p.tol and b["residual"] < p.tol
        t += p.dt
    zm, km = sm.state()
    zf, kf = sf.state()
    assert rel_err(zm, zf) < 1e-8
    assert rel_err(km, kf) < 1e-8
    sm.close()
    sf.close()


def test_128_cube_against_oracle():
    """The largest workload (the 128^3 cube: 25,264,128 face rows, 176M
    nonzeros) against the oracle for one step: the FP64 form and the mixed
    form both solved to 1e-13, face traces and cell values within 1e-10 of the
    oracle's, the CSR pattern bit-exact."""
    p = problems.diffusion3d(N=128, steps=1)
    s, m = _pair(p, check_every=8)
    pm = variant(p, form=L.FORM_MIXED)
    sm = problems.make_solver(pm, check_every=8)
    sm.setup(tol=1e-13, max_iter=20000, check_every=8, max_sweeps=60)
    assert s.F == 25264128 and s.C == 12582912
    a = s.step(0.0, p.dt)
    b = sm.step(0.0, p.dt)
    m.step(0.0, p.dt, 1e-13)
    assert a["residual"] < 1e-13 and b["residual"] < 1e-13
    for sv in (s, sm):
        zf, zk = sv.state()
        assert rel_err(zf, m.Z_iF) < TOL_STATE
        assert rel_err(zk, m.Z_iK) < TOL_STATE
    sm.close()
    rowptr, cols, _, _ = s.system()
    assert np.array_equal(rowptr, m.rowptr) and np.array_equal(cols, m.cols)
    s.close()


def test_mixed_fp32_matrix_is_the_rounded_fp64_matrix():
    """The mixed form's FP32 copy of the assembled values (converted on the
    integer pipes) equals the FP64 values rounded to nearest even, bit for
    bit, over the 32^3 tetrahedral system (1.3M values) and the two-component
    triangle system."""
    for p in (problems.diffusion3d(N=32, steps=1, form=L.FORM_MIXED), problems.adr2d(N=32, steps=1, form=L.FORM_MIXED)):
        s = problems.make_solver(p)
        s.preIterate(0.0, p.dt)
        s.assembleLinearSystem(0.0, p.dt)
        _, _, vals, _ = s.system()
        v32 = s.system32()
        assert v32.dtype == np.float32 and v32.size == vals.size
        assert np.array_equal(v32.view(np.uint32), vals.astype(np.float32).view(np.uint32)), p.name
        s.close()


def test_mixed_precision_matches_fp64_oracle():
    """FP32 inner BiCGStab + FP64 refinement to 1e-10: error vs the FP64 oracle."""
    p = problems.diffusion3d(N=12, steps=3, form=L.FORM_MIXED)
    s = problems.make_solver(p)
    m = OracleModel.from_problem(p)
    t = 0.0
    for _ in range(p.steps):
        st = s.step(t, p.dt)
        m.step(t, p.dt, 1e-13)
        assert st["sweeps"] >= 1 and st["residual"] < p.tol
        t += p.dt
    zf, zk = s.state()
    assert rel_err(zf, m.Z_iF) < 1e-8
    assert rel_err(zk, m.Z_iK) < 1e-8
    s.close()


def test_deterministic():
    p = problems.diffusion3d(N=8, steps=2)
    outs = []
    for _ in range(2):
        s = problems.make_solver(p)
        t = 0.0
        for _ in range(p.steps):
            s.step(t, p.dt)
            t += p.dt
        outs.append(s.state())
        s.close()
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def test_not_converged_is_reported():
    p = problems.diffusion3d(N=6, steps=1)
    s = problems.make_solver(p)
    s.setup(tol=1e-14, max_iter=1, check_every=1)
    with pytest.raises(L.MhfemError) as ei:
        s.step(0.0, p.dt)
    assert ei.value.status == L.ERR_NOT_CONVERGED
    s.close()


def test_nan_coefficient_is_reported():
    p = problems.diffusion3d(N=4, steps=1)
    D = np.array(p.coeffs["D"], copy=True)
    D[5] = np.nan
    s = problems.make_solver(p)
    s.set_coeff("D", D)
    with pytest.raises(L.MhfemError) as ei:
        s.step(0.0, p.dt)
    assert ei.value.status in (L.ERR_NONPOSITIVE_DIAGONAL, L.ERR_NOT_FINITE)
    s.close()


def test_box_vertex_order_is_checked():
    """Box cells must be axis-aligned with their vertices counterclockwise from
    the lowest corner (the closed-form mass matrix reads the side lengths and
    face orientations from that order): another order is refused at
    mhfem_set_mesh with an error, not solved wrongly."""
    from mhfem import meshgen
    from mhfem.solver import Solver, StaticConfig

    for dim in (2, 3):
        coords, cells = meshgen.square_rectangles(4) if dim == 2 else meshgen.cube_cuboids(3)
        rot = [1, 2, 3, 0] if dim == 2 else [1, 2, 3, 0, 5, 6, 7, 4]
        s = Solver(StaticConfig(dim=dim, n_eq=1, cell=L.CELL_BOX))
        with pytest.raises(L.MhfemError) as ei:
            s.setMesh(coords, cells[:, rot])
        assert ei.value.status == L.ERR_INVALID_ARGUMENT
        s.setMesh(coords, cells)  # the canonical order is accepted
        s.close()


GMRES_CASES = ["heat2d", "diffusion3d", "adr2d", "diffusion3d_box", "adr2d_rect_implicit_upwind", "diffusion3d_n3"]


@pytest.mark.parametrize("variant", ["cgs", "cgsr"])
@pytest.mark.parametrize("name", GMRES_CASES)
def test_gmres_step_parity(name, variant):
    """Restarted GMRES (the reference example's linear-solver = gmres) to a
    relative residual of 1e-13: face traces and cell values within 1e-10 of
    the oracle after every step, like the BiCGStab form."""
    p = CASES[name]
    s, m = _pair(p)
    s.setup(tol=1e-13, max_iter=20000, check_every=4, linear_solver="gmres", gmres_restart=30,
            gmres_variant=variant)
    t = 0.0
    for step in range(p.steps):
        st = s.step(t, p.dt)
        m.step(t, p.dt, 1e-13)
        zf, zk = s.state()
        assert st["residual"] < 1e-13 and st["iterations"] > 0
        assert rel_err(zf, m.Z_iF) < TOL_STATE, f"step {step}: Z_iF"
        assert rel_err(zk, m.Z_iK) < TOL_STATE, f"step {step}: Z_iK"
        t += p.dt
    s.close()


def test_gmres_heat2d_full_size():
    """The 128^2 heat-equation workload with the reference example's solver
    keys (GMRES, CGS, restart 30), 3 steps against the oracle at the 1e-10
    bar; both solves run to 1e-13 like every other parity test."""
    p = problems.heat2d(N=128, steps=3)
    s, m = _pair(p, check_every=8)
    s.setup(tol=1e-13, max_iter=20000, check_every=8, linear_solver="gmres", gmres_restart=30, gmres_variant="cgs")
    t = 0.0
    for _ in range(p.steps):
        st = s.step(t, p.dt)
        m.step(t, p.dt, 1e-13)
        assert st["residual"] < 1e-13
        t += p.dt
    zf, zk = s.state()
    assert rel_err(zf, m.Z_iF) < TOL_STATE
    assert rel_err(zk, m.Z_iK) < TOL_STATE
    s.close()


def test_gmres_adaptive_restart_full_size():
    """The reference example's adaptive restart keys (gmres-restarting-min 3,
    -max 30, -step-min 2, -step-max 4) on the 128^2 heat-equation workload
    and on the 512^2 ADR workload: every step's face traces and cell values
    within 1e-10 of the oracle, as with the fixed restart length."""
    for p in (problems.heat2d(N=128, steps=3), problems.adr2d(N=512, steps=2)):
        s, m = _pair(p, check_every=8)
        s.setup(tol=1e-13, max_iter=20000, check_every=8, linear_solver="gmres", gmres_restart=30,
                gmres_variant="cgs", gmres_restart_min=3, gmres_restart_step_min=2, gmres_restart_step_max=4)
        t = 0.0
        for _ in range(p.steps):
            st = s.step(t, p.dt)
            m.step(t, p.dt, 1e-13)
            assert st["residual"] < 1e-13
            t += p.dt
        zf, zk = s.state()
        assert rel_err(zf, m.Z_iF) < TOL_STATE, p.name
        assert rel_err(zk, m.Z_iK) < TOL_STATE, p.name
        s.close()


def test_gmres_not_converged_is_reported():
    p = problems.diffusion3d(N=6, steps=1)
    s = problems.make_solver(p)
    s.setup(tol=1e-14, max_iter=3, check_every=1, linear_solver="gmres", gmres_restart=2)
    with pytest.raises(L.MhfemError) as ei:
        s.step(0.0, p.dt)
    assert ei.value.status == L.ERR_NOT_CONVERGED
    s.close()
