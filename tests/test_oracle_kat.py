"""Known-answer tests that pin the CPU oracle (no GPU needed).

The reference ships no tests or golden vectors and cannot be built here, so
the oracle is pinned to answers that follow from mathematics and from the
reference's own definitions:

1. the stored b_ijK is the inverse of the RT0 mass matrix
   int_K phi_e . phi_f dx with the basis of BasisFunctions_RTN0.h:32-51,
   phi_e(x) = (x - v_e) / (d |K|), integrated exactly (degree-2 rules);
2. linear patch test: a linear field with matching Dirichlet data is
   reproduced exactly (to rounding) by the hybridized RT0 scheme;
3. local conservation: sum_e v_Ke = |K| f - |K| N (Z_K^new - Z_K^old) / tau;
4. row structure: unit diagonal, ascending columns, row lengths (2f-1)n /
   1 / f n (LinearSystem.h:26-34, BoundaryConditions.hpp:283-299);
5. the oracle's BiCGStab agrees with a direct sparse solve.
"""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

from helpers import golden_case, golden_names, rel_err, small_cases, variant
from mhfem import _lib as L
from mhfem import meshgen, problems
from oracle.oracle import OracleModel, build_faces

pytestmark = []


def _quad_mass(X):
    """Exact int_K phi_e . phi_f for a simplex with vertices X [nf][d]."""
    nf, d = X.shape
    if d == 2:
        area = 0.5 * abs(np.linalg.det(X[1:] - X[0]))
        pts = [(X[a] + X[b]) / 2 for a, b in [(0, 1), (1, 2), (0, 2)]]
        wts = [area / 3] * 3
        meas = area
    else:
        vol = abs(np.linalg.det(X[1:] - X[0])) / 6
        al, be = 0.5854101966249685, 0.1381966011250105
        pts = []
        for k in range(4):
            lam = np.full(4, be)
            lam[k] = al
            pts.append(lam @ X)
        wts = [vol / 4] * 4
        meas = vol
    M = np.zeros((nf, nf))
    for x, w in zip(pts, wts):
        phi = [(x - X[e]) / (d * meas) for e in range(nf)]
        for e in range(nf):
            for f in range(nf):
                M[e, f] += w * phi[e] @ phi[f]
    return M


def _unpack(bK, nf):
    B = np.zeros((nf, nf))
    for f in range(nf):
        for e in range(f + 1):
            B[e, f] = B[f, e] = bK[e + f * (f + 1) // 2]
    return B


@pytest.mark.parametrize("dim", [2, 3])
def test_mass_matrix_is_inverse_of_rt0_quadrature(dim):
    p = problems.heat2d(N=4) if dim == 2 else problems.diffusion3d(N=2)
    p.coeffs["D"] = 1.0
    m = OracleModel.from_problem(p)
    m.pre_iterate(0.0, p.dt)
    nf, S, C = dim + 1, m.S, m.C
    b = m.b.reshape(S, C)
    for K in range(0, C, max(1, C // 7)):
        X = p.coords[p.cells[K]]
        Binv = _unpack(b[:, K], nf)
        M = _quad_mass(X)
        assert np.abs(Binv @ M - np.eye(nf)).max() < 1e-11
        # stored row sums (MassMatrix.h:594-597)
        assert np.allclose(b[S - nf:, K], Binv.sum(axis=1), rtol=1e-14, atol=0)


@pytest.mark.parametrize("dim", [2, 3])
def test_lumped_mass_matrix_is_spd(dim):
    p = problems.heat2d(N=4) if dim == 2 else problems.diffusion3d(N=2)
    p.config.mass_lumping = True
    m = OracleModel.from_problem(p)
    m.pre_iterate(0.0, p.dt)
    nf, S, C = dim + 1, m.S, m.C
    b = m.b.reshape(S, C)
    for K in range(C):
        B = _unpack(b[:, K], nf)
        assert np.linalg.eigvalsh(B).min() > 0


def _linear_problem(dim, neumann_sign=None, box=False, lumping=False):
    c = np.array([0.7, -0.4, 0.25][:dim])
    c0 = 0.3
    Dval = 2.5
    if box:
        coords, cells = meshgen.square_rectangles(6) if dim == 2 else meshgen.cube_cuboids(4)
    elif dim == 2:
        coords, cells = meshgen.square_triangles(6, 0.2, 99)
    else:
        coords, cells = meshgen.cube_tetrahedra(3, 0.15, 99)
    cen = meshgen.cell_centroids(coords, cells)
    Z0 = cen @ c + c0

    def bc_fn(fv, fc):
        F = fc.shape[0]
        fcen = meshgen.face_centroids(coords, fv)
        tags = np.zeros(F, np.uint8)
        vals = np.zeros(F)
        bnd = fc[:, 1] < 0
        if neumann_sign is not None:
            right = bnd & (np.abs(fcen[:, 0] - 1.0) < 1e-12)
            tags[right] = problems.BC_FIXED_FLUX
            # outward normal of the face x = 1 is +e_x
            vals[right] = neumann_sign * Dval * c[0]
        return tags, vals, fcen @ c + c0

    cfg = problems.StaticConfig(dim=dim, n_eq=1, mass_lumping=lumping, cell=L.CELL_BOX if box else L.CELL_SIMPLEX)
    coeffs = {"N": 1.0, "u": 0.0, "m": 1.0, "D": Dval, "w": 0.0, "a": 0.0, "r": 0.0, "f": 0.0, "m_upw": 1.0,
              "m_bnd": 1.0}
    p = problems.Problem("linear", cfg, coords, cells, coeffs, Z0, 1e-2, 3, 1e-13, bc_fn, 0)
    return p, c, c0


@pytest.mark.parametrize("dim", [2, 3])
def test_linear_patch_dirichlet(dim):
    p, c, c0 = _linear_problem(dim)
    m = OracleModel.from_problem(p)
    t = 0.0
    for _ in range(p.steps):
        m.step(t, p.dt, 1e-14)
        t += p.dt
    fcen = meshgen.face_centroids(p.coords, m.face_verts)
    assert rel_err(m.Z_iF, fcen @ c + c0) < 1e-11
    assert rel_err(m.Z_iK, meshgen.cell_centroids(p.coords, p.cells) @ c + c0) < 1e-11


@pytest.mark.parametrize("dim", [2, 3])
def test_linear_patch_neumann(dim):
    """FixedFlux J on x = 1.  With the right-hand side -J |E| of the reference's
    row setter (BoundaryConditions.hpp:413-418) the prescribed J is the outward
    normal component of the velocity v = -D grad Z: J = -D grad Z . n."""
    p, c, c0 = _linear_problem(dim, neumann_sign=-1.0)
    m = OracleModel.from_problem(p)
    t = 0.0
    for _ in range(p.steps):
        m.step(t, p.dt, 1e-14)
        t += p.dt
    fcen = meshgen.face_centroids(p.coords, m.face_verts)
    assert rel_err(m.Z_iF, fcen @ c + c0) < 1e-10


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("lumping", [False, True])
def test_linear_patch_boxes(dim, lumping):
    """Rectangles and cuboids (graded, so not squares or cubes), with and
    without lumping: the RT0 scheme of MassMatrix.h:152-508 reproduces a
    linear solution, under Dirichlet data and under a prescribed flux."""
    for sign in (None, -1.0):
        p, c, c0 = _linear_problem(dim, neumann_sign=sign, box=True, lumping=lumping)
        m = OracleModel.from_problem(p)
        t = 0.0
        for _ in range(p.steps):
            m.step(t, p.dt, 1e-14)
            t += p.dt
        fcen = meshgen.face_centroids(p.coords, m.face_verts)
        assert rel_err(m.Z_iF, fcen @ c + c0) < 1e-10
        assert rel_err(m.Z_iK, meshgen.cell_centroids(p.coords, p.cells) @ c + c0) < 1e-10


def test_box_topology():
    """Face numbering of box cells: first appearance over (cell, local face)
    with the local faces of the reference's Quadrangle / Hexahedron; every
    interior face has two cells; face counts of the tensor grids."""
    for dim, N in ((2, 3), (3, 2)):
        coords, cells = meshgen.square_rectangles(N) if dim == 2 else meshgen.cube_cuboids(N)
        fv, fc, cf = build_faces(dim, cells, 1)
        F = fc.shape[0]
        expect = 2 * N * (N + 1) if dim == 2 else 3 * N * N * (N + 1)
        assert F == expect
        assert (fc[:, 1] >= 0).sum() == (2 * N * (N - 1) if dim == 2 else 3 * N * N * (N - 1))
        assert np.array_equal(cf[0], np.arange(2 * dim))  # the first cell numbers its faces 0..nf-1
        # face e of cell 0 lies on the side the reference names it after
        fcen = meshgen.face_centroids(coords, fv)
        ccen = coords[cells[0]].mean(axis=0)
        d = fcen[cf[0]] - ccen
        if dim == 2:  # bottom, right, top, left
            assert d[0, 1] < 0 and d[1, 0] > 0 and d[2, 1] > 0 and d[3, 0] < 0
        else:  # bottom, front, right, back, left, top
            assert d[0, 2] < 0 and d[1, 1] < 0 and d[2, 0] > 0 and d[3, 1] > 0 and d[4, 0] < 0 and d[5, 2] > 0


def test_local_conservation():
    p = problems.diffusion3d(N=3, steps=1)
    p = variant(p, mobility_upwind=True, coeffs={"f": 0.7})
    m = OracleModel.from_problem(p)
    z_old = m.Z_iK.copy()
    m.step(0.0, p.dt, 1e-14)
    C, nf = m.C, 4
    v = m.v_iKe.reshape(nf, C)
    X = p.coords[p.cells]
    vol = np.abs(np.linalg.det(X[:, 1:] - X[:, :1])) / 6
    balance = v.sum(axis=0) - (vol * 0.7 - vol * (m.Z_iK - z_old) / p.dt)
    assert np.abs(balance).max() < 1e-10 * max(1.0, np.abs(v).max())


@pytest.mark.parametrize("name", sorted(small_cases()))
def test_row_structure_and_direct_solve(name):
    p = small_cases()[name]
    m = OracleModel.from_problem(p)
    m.pre_iterate(0.0, p.dt)
    m.assemble(0.0, p.dt)
    A = m.csr()
    n, nf = p.n, p.config.faces_per_cell
    lens = np.diff(A.indptr)
    interior = np.repeat(m.face_cells[:, 1] >= 0, n)
    assert np.all(lens[interior] == (2 * nf - 1) * n)
    tags = m.tags.reshape(n, m.F).T.ravel()  # row order E*n + i
    bnd = ~interior
    assert np.all(lens[bnd & (tags == 0)] == 1)
    assert np.all(lens[bnd & (tags != 0)] == nf * n)
    for r in range(A.shape[0]):
        cols = A.indices[A.indptr[r]:A.indptr[r + 1]]
        assert np.all(np.diff(cols) > 0)
    assert np.all(A.diagonal() == 1.0)
    x = spla.spsolve(A.tocsc(), m.rhs)
    m.solve(1e-14)
    assert rel_err(m.Z_iF, x) < 1e-10


@pytest.mark.parametrize("name", golden_names())
def test_oracle_reproduces_golden(name):
    """The oracle still gives the committed fixtures (tests/golden): topology
    and CSR pattern bit-exact, the first step's local arrays and system within
    1e-12, the states after every step within 1e-10 (the solves run to 1e-13;
    the fixtures were written with one thread, the test uses all)."""
    p, d = golden_case(name)
    m = OracleModel.from_problem(p)
    assert np.array_equal(m.face_verts, d["face_verts"])
    assert np.array_equal(m.face_cells, d["face_cells"])
    assert np.array_equal(m.cell_faces, d["cell_faces"])
    t = 0.0
    for step in range(p.steps):
        m.pre_iterate(t, p.dt)
        m.assemble(t, p.dt)
        if step == 0:
            assert np.array_equal(m.rowptr, d["rowptr"]) and np.array_equal(m.cols, d["cols"])
            for got, key in ((m.b, "b0"), (m.R_ijKe, "R_ijKe0"), (m.R_iK, "R_iK0"), (m.vals, "vals0"),
                             (m.rhs, "rhs0")):
                assert rel_err(got, d[key]) < 1e-12, key
        m.solve(1e-13)
        m.post_iterate(t, p.dt)
        assert rel_err(m.Z_iF, d["Z_iF"][step]) < 1e-10, f"step {step}: Z_iF"
        assert rel_err(m.Z_iK, d["Z_iK"][step]) < 1e-10, f"step {step}: Z_iK"
        t += p.dt


@pytest.mark.parametrize("name,lumping", [("heat2d", False), ("heat2d", True), ("diffusion3d", False),
                                          ("diffusion3d", True), ("diffusion3d_box", False)])
def test_pure_diffusion_matrix_is_symmetric_before_row_scaling(name, lumping):
    """For pure diffusion the assembled A is symmetric before the unit-diagonal
    row scaling, so the stored rows a_EF = A_EF / d_E satisfy
    a_EF d_E = a_FE d_F for one positive d over every pair of rows that are
    not Dirichlet rows (a Dirichlet row keeps only its diagonal).  d is
    propagated along the graph from one row per component and the relation
    checked on every pair."""
    small = {"heat2d": dict(N=6), "diffusion3d": dict(N=3), "diffusion3d_box": dict(N=3)}[name]
    p = variant(problems.WORKLOADS[name](steps=1, **small), mass_lumping=lumping)
    m = OracleModel.from_problem(p)
    m.pre_iterate(0.0, p.dt)
    m.assemble(0.0, p.dt)
    A = m.csr().tocsr()
    R = A.shape[0]
    # n = 1: row index = face index; tags matter on boundary faces only
    free = (m.face_cells[:, 1] >= 0) | (m.tags != 0)
    a = {}
    for r in np.flatnonzero(free):
        for k in range(A.indptr[r], A.indptr[r + 1]):
            c = A.indices[k]
            if c != r and free[c]:
                a[(r, c)] = A.data[k]
    assert a, "no coupled free rows"
    for (r, c), v in a.items():
        assert (r, c)[::-1] in a, f"entry ({r}, {c}) has no transposed partner"
        assert v * a[(c, r)] > 0
    nbr = {}
    for r, c in a:
        nbr.setdefault(r, []).append(c)
    d = np.full(R, np.nan)
    for root in nbr:
        if not np.isnan(d[root]):
            continue
        d[root] = 1.0
        stack = [root]
        while stack:
            r = stack.pop()
            for c in nbr[r]:
                if np.isnan(d[c]):
                    d[c] = d[r] * a[(r, c)] / a[(c, r)]
                    stack.append(c)
    scale = max(abs(v * d[r]) for (r, c), v in a.items())
    worst = max(abs(v * d[r] - a[(c, r)] * d[c]) for (r, c), v in a.items())
    assert worst < 1e-12 * scale


def test_same_seed_same_mesh_numbering_and_system():
    """Determinism: the same seeds give an identical mesh, face numbering,
    CSR pattern and (one thread) bitwise identical values."""
    def run():
        p = problems.diffusion3d(N=3, steps=1)
        m = OracleModel.from_problem(p, threads=1)
        m.pre_iterate(0.0, p.dt)
        m.assemble(0.0, p.dt)
        return p, m

    (p1, m1), (p2, m2) = run(), run()
    assert np.array_equal(p1.coords, p2.coords) and np.array_equal(p1.cells, p2.cells)
    assert np.array_equal(np.asarray(p1.coeffs["D"]), np.asarray(p2.coeffs["D"]))
    for k in ("face_verts", "face_cells", "cell_faces", "rowptr", "cols", "vals", "rhs"):
        assert np.array_equal(getattr(m1, k), getattr(m2, k)), k


@pytest.mark.parametrize("name", ["diffusion3d_dummy_row", "diffusion3d_n2_dummy_row"])
def test_dummy_equation_for_singular_q(name):
    """Cells whose Q_K has an all-zero row i take the reference's dummy
    equation Q_ii = 1, R_iK += Z_iK (Solver.hpp:829-847).  There D_ij = 0 and
    N_ij = 0 for that i, so b and hence R_ijKe vanish, and the reconstruction
    Z_iK = sum R_ijKf Z_jF + R_iK (Solver.hpp:1283-1292) gives, whatever the
    face traces, Z_iK_new = Z_iK + |K| f_i - sum_e m_iE_upw w_iKe (the R_iK of
    SecondaryCoefficients.h:87-127 without its N and advection terms).  The
    other cells still follow the face solve, checked against a direct sparse
    solve."""
    p = small_cases()[name]
    m = OracleModel.from_problem(p)
    n, C = p.n, p.C
    iso = p.extra["dummy_cells"]
    i = p.extra.get("dummy_component", 0)
    X = p.coords[p.cells]
    vol = np.abs(np.linalg.det(X[:, 1:] - X[:, :1])) / 6
    f = np.broadcast_to(np.asarray(p.coeffs.get("f", 0.0), np.float64), (n * C,)).reshape(n, C)
    w = np.asarray(p.coeffs["w"], np.float64).reshape(n, 4, C)
    t = 0.0
    for _ in range(p.steps):
        z_old = m.Z_iK.reshape(n, C)[i, iso].copy()
        m.pre_iterate(t, p.dt)
        m.assemble(t, p.dt)
        x = spla.spsolve(m.csr().tocsc(), m.rhs)
        m.solve(1e-14)
        assert rel_err(m.Z_iF, x) < 1e-10
        m.post_iterate(t, p.dt)
        expect = z_old + vol[iso] * f[i, iso] - w[i, :, iso].sum(axis=1)
        got = m.Z_iK.reshape(n, C)[i, iso]
        assert np.abs(got - expect).max() <= 1e-13 * max(1.0, np.abs(expect).max())
        t += p.dt
