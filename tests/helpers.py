"""Shared helpers: model variants and GPU-vs-oracle comparison."""
from __future__ import annotations

import copy
from pathlib import Path

import numpy as np

from mhfem import _lib as L
from mhfem import meshgen, problems
from mhfem.solver import StaticConfig

GOLDEN = Path(__file__).resolve().parent / "golden"


def rel_err(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = max(np.abs(b).max(initial=0.0), 1e-300)
    return float(np.abs(a - b).max(initial=0.0) / scale)


def variant(p: problems.Problem, **changes) -> problems.Problem:
    q = copy.copy(p)
    q.config = copy.copy(p.config)
    q.coeffs = dict(p.coeffs)
    for k, v in changes.items():
        if hasattr(q.config, k):
            setattr(q.config, k, v)
        elif k == "coeffs":
            q.coeffs.update(v)
        else:
            setattr(q, k, v)
    return q


def small_cases():
    """Small models that together exercise every branch of the path."""
    cases = {}
    cases["heat2d"] = problems.heat2d(N=8, steps=3)
    cases["diffusion3d"] = problems.diffusion3d(N=4, steps=3)
    cases["adr2d"] = problems.adr2d(N=8, steps=3)
    cases["diffusion3d_lumped"] = variant(problems.diffusion3d(N=4, steps=2), mass_lumping=True)
    cases["heat2d_lumped"] = variant(problems.heat2d(N=8, steps=2), mass_lumping=True)
    # mobility upwind with a heterogeneous mobility (K6 and K13 active)
    p = problems.diffusion3d(N=4, steps=3)
    rng = np.random.default_rng(7)
    cases["diffusion3d_mobility"] = variant(p, mobility_upwind=True,
                                            coeffs={"m": rng.uniform(0.5, 2.0, p.C), "m_bnd": 1.5})
    p = problems.adr2d(N=8, steps=3)
    cases["adr2d_implicit_upwind"] = variant(p, advection=L.IMPLICIT_UPWIND)
    # the trace discretization needs a low cell Peclet number for a positive diagonal
    cases["adr2d_implicit_trace"] = variant(p, advection=L.IMPLICIT_TRACE,
                                            coeffs={"a": np.asarray(p.coeffs["a"]) * 0.02})
    cases["adr2d_mobility"] = variant(p, mobility_upwind=True,
                                      coeffs={"m": np.random.default_rng(3).uniform(0.5, 2.0, 2 * p.C)})
    cases["diffusion3d_n2"] = diffusion3d_n2(3)
    cases.update(three_component_cases())
    cases.update(box_cases())
    cases.update(dummy_row_cases())
    return cases


def diffusion3d_n2(N: int, steps: int = 2) -> problems.Problem:
    """Two components on tetrahedra with coupled reaction and a full w field."""
    p3 = problems.diffusion3d(N=N, steps=steps)
    C = p3.C
    rng = np.random.default_rng(11)
    Nc = np.zeros((2, 2, C)); Nc[0, 0] = 1.0; Nc[1, 1] = 2.0
    D = np.zeros((2, 2, C)); D[0, 0] = p3.coeffs["D"]; D[1, 1] = 0.5 * p3.coeffs["D"]; D[0, 1] = 0.1
    r = np.zeros((2, 2, C)); r[0, 0] = 0.3; r[0, 1] = -0.1; r[1, 0] = -0.1; r[1, 1] = 0.2
    w = rng.uniform(-0.01, 0.01, (2, 4, C))
    base_bc = p3.bc_fn

    def bc2(fv, fc):
        t, v, d = base_bc(fv, fc)
        F = fc.shape[0]
        return np.concatenate([t, t]), np.concatenate([v, v + 0.1 * (t == 1)]), np.concatenate([d + 0.2, d])

    q = variant(p3, n_eq=2, coeffs={"N": Nc.ravel(), "D": D.ravel(), "r": r.ravel(), "w": w.ravel(), "f": 0.5})
    q.bc_fn = bc2
    q.Z0 = rng.uniform(0, 1, 2 * C)
    return q


def isolated_interior_cells(cells: np.ndarray, stride: int = 5) -> np.ndarray:
    """Simplex cells with no boundary face, no two of them sharing a face:
    every `stride`-th interior cell in index order, skipping the neighbours of
    cells already taken."""
    C, nf = cells.shape
    faces = np.sort(np.stack([np.delete(cells, e, axis=1) for e in range(nf)], axis=1), axis=2)
    _, inv, counts = np.unique(faces.reshape(C * nf, -1), axis=0, return_inverse=True, return_counts=True)
    inv = inv.reshape(C, nf)
    interior = (counts[inv] == 2).all(axis=1)
    by_face = {}
    for K in range(C):
        for e in range(nf):
            by_face.setdefault(int(inv[K, e]), []).append(K)
    taken, blocked = [], set()
    for K in np.flatnonzero(interior)[::stride]:
        if K in blocked:
            continue
        taken.append(int(K))
        for e in range(nf):
            blocked.update(by_face[int(inv[K, e])])
    return np.array(taken, np.int64)


def dummy_row_cases(N: int = 4):
    """Cells whose local matrix Q_K has an all-zero row, so that the reference
    replaces that row by the dummy equation Q_ii = 1, R_iK += Z_iK
    (Solver.hpp:829-847): on isolated interior cells one component has D = 0,
    N = 0 and r = 0 (and u = 0, no implicit advection).  Its face rows there
    take their entries from the neighbouring cells only.  n = 1 on tetrahedra,
    and n = 2 on tetrahedra where only the second component vanishes (the
    first keeps its coupling D_01, so the LU of Q mixes the dummy row into
    the other one)."""
    cases = {}
    p = problems.diffusion3d(N=N, steps=3)
    C = p.C
    iso = isolated_interior_cells(p.cells)
    rng = np.random.default_rng(23)
    D = np.array(p.coeffs["D"], np.float64, copy=True)
    D[iso] = 0.0
    Nc = np.ones(C)
    Nc[iso] = 0.0
    w = rng.uniform(-0.01, 0.01, (4, C))
    q = variant(p, coeffs={"D": D, "N": Nc, "w": w.ravel()})
    q.Z0 = rng.uniform(0, 1, C)
    q.extra = {"dummy_cells": iso}
    cases["diffusion3d_dummy_row"] = q

    p3 = problems.diffusion3d(N=N, steps=3)
    Nc = np.zeros((2, 2, C)); Nc[0, 0] = 1.0; Nc[1, 1] = 2.0
    D = np.zeros((2, 2, C)); D[0, 0] = p3.coeffs["D"]; D[1, 1] = 0.5 * p3.coeffs["D"]
    D[0, 1] = 0.1; D[1, 0] = 0.05
    r = np.zeros((2, 2, C)); r[0, 0] = 0.3; r[0, 1] = -0.1; r[1, 0] = -0.1; r[1, 1] = 0.2
    for arr in (Nc, D, r):
        arr[1, :, iso] = 0.0
    w = rng.uniform(-0.01, 0.01, (2, 4, C))
    base_bc = p3.bc_fn

    def bc2(fv, fc):
        t, v, d = base_bc(fv, fc)
        return np.concatenate([t, t]), np.concatenate([v, v + 0.1 * (t == 1)]), np.concatenate([d + 0.2, d])

    q = variant(p3, n_eq=2, coeffs={"N": Nc.ravel(), "D": D.ravel(), "r": r.ravel(), "w": w.ravel(), "f": 0.5})
    q.bc_fn = bc2
    q.Z0 = rng.uniform(0, 1, 2 * C)
    q.extra = {"dummy_cells": iso, "dummy_component": 1}
    cases["diffusion3d_n2_dummy_row"] = q
    return cases


def box_cases():
    """Rectangles and cuboids: full and lumped RT0 mass matrices, mobility
    upwinding (reconstructed velocities), advection on rectangles (explicit and
    implicit upwind, two components) and two coupled components on cuboids."""
    cases = {}
    cases["heat2d_rect"] = problems.heat2d_rect(N=8, steps=3)
    cases["heat2d_rect_lumped"] = problems.heat2d_rect(N=8, steps=2, lumping=True)
    cases["diffusion3d_box"] = problems.diffusion3d_box(N=4, steps=3)
    cases["diffusion3d_box_lumped"] = problems.diffusion3d_box(N=4, steps=2, lumping=True)
    p = problems.diffusion3d_box(N=4, steps=3)
    rng = np.random.default_rng(17)
    cases["diffusion3d_box_mobility"] = variant(p, mobility_upwind=True,
                                                coeffs={"m": rng.uniform(0.5, 2.0, p.C), "m_bnd": 1.5})
    p = problems.adr2d(N=8, steps=3, box=True)
    cases["adr2d_rect"] = p
    cases["adr2d_rect_implicit_upwind"] = variant(p, advection=L.IMPLICIT_UPWIND, mass_lumping=False)
    # two components on cuboids: coupled diffusion and reaction, a full w field
    p3 = problems.diffusion3d_box(N=3, steps=2)
    C = p3.C
    Nc = np.zeros((2, 2, C)); Nc[0, 0] = 1.0; Nc[1, 1] = 2.0
    D = np.zeros((2, 2, C)); D[0, 0] = p3.coeffs["D"]; D[1, 1] = 0.5 * p3.coeffs["D"]; D[0, 1] = 0.1
    r = np.zeros((2, 2, C)); r[0, 0] = 0.3; r[0, 1] = -0.1; r[1, 0] = -0.1; r[1, 1] = 0.2
    w = rng.uniform(-0.01, 0.01, (2, 6, C))
    base_bc = p3.bc_fn

    def bc2(fv, fc):
        t, v, d = base_bc(fv, fc)
        return np.concatenate([t, t]), np.concatenate([v, v + 0.1 * (t == 1)]), np.concatenate([d + 0.2, d])

    q = variant(p3, n_eq=2, coeffs={"N": Nc.ravel(), "D": D.ravel(), "r": r.ravel(), "w": w.ravel(), "f": 0.5})
    q.bc_fn = bc2
    q.Z0 = rng.uniform(0, 1, 2 * C)
    cases["diffusion3d_box_n2"] = q
    return cases


def three_component_cases():
    """n = 3: tetrahedra with coupled diffusion, reaction and a w field; triangles
    with advection on every component (implicit upwind) and coupled reaction."""
    cases = {}
    n = 3
    p = problems.diffusion3d(N=3, steps=2)
    C = p.C
    rng = np.random.default_rng(13)
    Nc = np.zeros((n, n, C))
    D = np.zeros((n, n, C))
    for i in range(n):
        Nc[i, i] = 1.0 + i
        D[i, i] = (1.0, 0.5, 2.0)[i] * p.coeffs["D"]
    D[0, 1] = 0.1
    D[1, 2] = 0.05
    r = np.zeros((n, n, C))
    r[0, 0], r[1, 1], r[2, 2] = 0.3, 0.2, 0.25
    r[0, 1] = r[1, 0] = -0.05
    r[1, 2] = r[2, 1] = -0.04
    w = rng.uniform(-0.01, 0.01, (n, 4, C))
    base_bc = p.bc_fn

    def bc3(fv, fc):
        t, v, d = base_bc(fv, fc)
        return (np.concatenate([t] * n), np.concatenate([v, v + 0.1 * (t == 1), v]),
                np.concatenate([d + 0.2, d, d + 0.1]))

    q = variant(p, n_eq=n, coeffs={"N": Nc.ravel(), "D": D.ravel(), "r": r.ravel(), "w": w.ravel(), "f": 0.5})
    q.bc_fn = bc3
    q.Z0 = rng.uniform(0, 1, n * C)
    cases["diffusion3d_n3"] = q

    p = problems.adr2d(N=6, steps=2)
    C = p.C
    nf = 3
    D2 = np.asarray(p.coeffs["D"]).reshape(2, 2, C)
    normals = meshgen.outward_face_normals(p.coords, p.cells)
    flux = np.einsum("cfd,d->fc", normals, np.array([1.0, 0.3]))
    Nc = np.zeros((n, n, C))
    D = np.zeros((n, n, C))
    a = np.zeros((n, n, nf, C))
    for i in range(n):
        Nc[i, i] = 1.0
        D[i, i] = D2[0, 0] * (1.0, 0.5, 0.8)[i]
        a[i, i] = flux * (1.0, 0.7, 1.2)[i]
    r = np.zeros((n, n, C))
    r[0, 0], r[1, 1], r[2, 2] = 0.1, 0.1, 0.15
    r[0, 1] = r[1, 0] = -0.05
    r[1, 2] = r[2, 1] = -0.03
    base_bc2 = p.bc_fn

    def bc_adr3(fv, fc):
        t, v, d = base_bc2(fv, fc)
        F = fc.shape[0]
        t0, d0 = t[:F], d[:F]
        return np.concatenate([t0] * n), np.zeros(n * F), np.concatenate([d0, 0.5 * d0, 0 * d0])

    q = variant(p, n_eq=n, advection=L.IMPLICIT_UPWIND,
                coeffs={"N": Nc.ravel(), "D": D.ravel(), "a": a.ravel(), "r": r.ravel()})
    q.bc_fn = bc_adr3
    q.Z0 = np.zeros(n * C)
    cases["adr2d_n3_implicit_upwind"] = q
    return cases


def _restrict(p: problems.Problem, keep) -> problems.Problem:
    """p on the cells `keep` only (n = 1; vertices renumbered in order of use)."""
    q = variant(p)
    cells = p.cells[keep]
    used, inv = np.unique(cells.ravel(), return_inverse=True)
    q.coords = p.coords[used]
    q.cells = inv.reshape(cells.shape).astype(p.cells.dtype)
    for k, v in p.coeffs.items():
        if np.ndim(v) and np.size(v) == p.C:
            q.coeffs[k] = np.asarray(v)[keep]
    q.Z0 = np.asarray(p.Z0)[keep]
    return q


def _flux_bc(values=0.5, dirichlet=1.0):
    """Every boundary face carries the flux `values` (FixedFlux) except the
    first face, a Dirichlet face with value `dirichlet`."""
    def bc_fn(face_verts, face_cells):
        F = face_cells.shape[0]
        tags = np.full(F, 1, np.uint8)
        tags[0] = 0
        vals = np.full(F, values)
        return tags, vals, np.full(F, dirichlet)
    return bc_fn


def minimal_cases():
    """The smallest meshes: one cell (every face on the boundary), including
    a system that is the identity (every face Dirichlet: no off-diagonal
    entry, ELL width 0), and the one-square / one-cube splits whose cells
    share faces; n = 2 on the two-triangle square."""
    cases = {}
    p = problems.heat2d(N=1, steps=3)
    q = _restrict(p, [0])

    def all_dirichlet(face_verts, face_cells):
        F = face_cells.shape[0]
        return np.zeros(F, np.uint8), np.zeros(F), np.linspace(-0.7, 1.1, F)
    q.bc_fn = all_dirichlet
    cases["one_triangle_dirichlet"] = q
    q = _restrict(p, [1])
    q.bc_fn = _flux_bc()
    cases["one_triangle"] = q
    q = problems.heat2d(N=1, steps=3)
    q.bc_fn = _flux_bc(-0.25, 0.5)
    cases["one_square"] = q
    p = problems.diffusion3d(N=1, steps=3)
    q = _restrict(p, [0])
    q.bc_fn = _flux_bc()
    cases["one_tetrahedron"] = q
    cases["one_cube"] = p
    q = problems.heat2d_rect(N=1, steps=3)
    q.bc_fn = _flux_bc()
    cases["one_rectangle"] = q
    q = problems.diffusion3d_box(N=1, steps=3)
    q.bc_fn = _flux_bc(0.25, -1.0)
    cases["one_cuboid"] = q
    cases["one_square_n2"] = problems.adr2d(N=1, steps=3)
    return cases


def golden_names():
    return sorted(f.stem for f in GOLDEN.glob("*.npz"))


def golden_case(name: str):
    """A committed fixture (tests/golden/make_golden.py): the problem its
    inputs define, solved to 1e-13, and its expected outputs."""
    d = dict(np.load(GOLDEN / f"{name}.npz"))
    dim, n, lumping, advection, cell = (int(v) for v in d["config"])
    cfg = StaticConfig(dim=dim, n_eq=n, mass_lumping=bool(lumping), advection=advection, mobility_upwind=False,
                       cell=cell)
    coeffs = {k[5:]: (float(v[0]) if v.size == 1 else v) for k, v in d.items() if k.startswith("coef_")}
    bc = (d["bc_tags"], d["bc_values"], d["bc_dirichlet"])
    p = problems.Problem(name, cfg, d["coords"], d["cells"], coeffs, d["Z0"], float(d["dt"]), int(d["steps"]),
                         1e-13, lambda fv, fc: bc, 0)
    return p, d
