"""The smallest meshes (tests/helpers.py: minimal_cases): one cell with every
face on the boundary, from the identity system of an all-Dirichlet triangle
(no off-diagonal entry, ELL width 0) to the single cuboid (width 5), the
one-square and one-cube splits whose cells share faces, and n = 2 on the
two-triangle square.

CPU: the oracle solves every case and holds each Dirichlet face at its value.
GPU: the FP64 BiCGStab, mixed-precision and GMRES paths, and the learned
form on the one-equation simplex meshes (training in every step, the network
and its gate over a graph of 0 to 6 neighbours per face, all inside one
128-face tile), against the oracle after every step, at the bars of
test_gpu_parity.py (face numbering and the pattern bit-exact, traces and cell
values within 1e-10, both sides solved to 1e-13).
"""
import numpy as np
import pytest

from helpers import minimal_cases, rel_err, variant
from mhfem import _lib as L
from mhfem import problems
from oracle.oracle import OracleModel

CASES = minimal_cases()
TOL_STATE = 1e-10


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_minimal_mesh(name):
    p = CASES[name]
    m = OracleModel.from_problem(p)
    fv = m.face_verts
    tags, _, dirichlet = p.bc_fn(fv, m.face_cells)
    t = 0.0
    for _ in range(p.steps):
        m.step(t, p.dt, 1e-13)
        t += p.dt
        assert np.isfinite(m.Z_iF).all() and np.isfinite(m.Z_iK).all()
    # BoundaryConditions.hpp:367-376: a FixedValue row (on a boundary face;
    # the tags of interior faces are not read) is the identity row with the
    # Dirichlet value on the right-hand side; Z_iF is (F, i), F-major
    n, F = p.n, m.F
    z = m.Z_iF.reshape(F, n)
    bnd = m.face_cells[:, 1] < 0
    for i in range(n):
        fixed = (tags[i * F:(i + 1) * F] == 0) & bnd
        assert np.allclose(z[fixed, i], dirichlet[i * F:(i + 1) * F][fixed], rtol=0, atol=1e-12)
    if name == "one_triangle_dirichlet":
        assert int(np.diff(m.rowptr).max()) == 1  # every row is its diagonal only


FORMS = {"fp64": L.FORM_FP64, "mixed": L.FORM_MIXED, "gmres": L.FORM_FP64, "learned": L.FORM_LEARNED}
# the learned form takes one equation on simplex cells
PAIRS = [(name, form) for name in sorted(CASES) for form in FORMS
         if form != "learned" or (CASES[name].n == 1 and CASES[name].config.cell == L.CELL_SIMPLEX)]


def _solver(p, form):
    q = variant(p, form=FORMS[form])
    q.tol = 1e-13
    s = problems.make_solver(q, check_every=4)
    opts = {"tol": 1e-13, "max_iter": 20000, "check_every": 4}
    if form == "mixed":
        opts["max_sweeps"] = 60
    if form == "gmres":
        opts.update(linear_solver="gmres", gmres_restart=30)
    s.setup(**opts)
    return q, s


@pytest.mark.gpu
@pytest.mark.parametrize("name,form", PAIRS)
def test_minimal_mesh_parity(name, form):
    q, s = _solver(CASES[name], form)
    m = OracleModel.from_problem(q)
    fv, fc, cf = s.topology()
    assert np.array_equal(fv, m.face_verts)
    assert np.array_equal(fc, m.face_cells)
    assert np.array_equal(cf, m.cell_faces)
    t = 0.0
    for step in range(q.steps):
        st = s.step(t, q.dt)
        m.step(t, q.dt, 1e-13)
        assert st["residual"] < 1e-13
        zf, zk = s.state()
        assert rel_err(zf, m.Z_iF) < TOL_STATE, f"step {step}: Z_iF"
        assert rel_err(zk, m.Z_iK) < TOL_STATE, f"step {step}: Z_iK"
        t += q.dt
    rowptr, cols, _, _ = s.system()
    assert np.array_equal(rowptr, m.rowptr) and np.array_equal(cols, m.cols)
    s.close()
