"""The benchmark workloads as model definitions (coefficients, BCs, IC).

Each builder returns a :class:`Problem`: the static configuration, a seeded
synthetic mesh, the coefficient arrays in the reference's CUDA layouts
(BaseModel.h:18-125; a scalar means a uniform coefficient,
UniformCoefficient.h), a boundary-condition builder (tags FixedValue=0,
FixedFlux=1, AdvectiveOutflow=2, FixedFluxNoAdvection=3; arrays indexed
i*F + E), the initial cell values and the time stepping.

* ``heat2d``      plain FP64 heat equation on a 128^2 triangle mesh
                  (n=1, D=1, Dirichlet 0, Gaussian bump, dt=1e-4, 100 steps, tol 1e-12);
* ``diffusion3d`` heterogeneous diffusion on a 64^3 cube grid split into
                  tetrahedra (D = exp(g), f = 1, Dirichlet 0 on x=0,1, zero flux
                  elsewhere, dt=1e-3, 50 steps, tol 1e-10);
* ``adr2d``       coupled two-component advection-diffusion-reaction on a
                  512^2 triangle mesh (lumped mass, explicit upwind);
* ``diffusion3d`` with N=128 and the mixed form is the large mixed-precision case;
* ``diffusion3d_source`` adds the time-modulated source
                  f = 1 + 0.5 sin(2 pi t / T) psi(x) used by the learned form;
* ``heat2d_rect`` / ``diffusion3d_box`` are the heat and diffusion models on
                  graded rectangles / cuboids (box cells); ``adr2d(box=True)``
                  the coupled model on rectangles.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Callable

import numpy as np

from . import _lib as L
from . import meshgen
from .solver import StaticConfig

BC_FIXED_VALUE, BC_FIXED_FLUX, BC_ADVECTIVE_OUTFLOW, BC_FIXED_FLUX_NO_ADVECTION = 0, 1, 2, 3


@dataclass
class Problem:
    name: str
    config: StaticConfig
    coords: np.ndarray
    cells: np.ndarray
    coeffs: dict
    Z0: np.ndarray
    dt: float
    steps: int
    tol: float
    bc_fn: Callable
    grid_N: int
    source: tuple | None = None  # (amplitude, period) of the time-modulated source
    extra: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return self.config.n_eq

    @property
    def C(self) -> int:
        return self.cells.shape[0]


def _boundary_sides(coords, face_verts, face_cells, dim):
    """For each face: which sides of the unit box it lies on (tolerance 1e-12)."""
    cen = meshgen.face_centroids(coords, face_verts)
    bnd = face_cells[:, 1] < 0
    sides = {}
    for d, name in enumerate("xyz"[:dim]):
        sides[name + "0"] = bnd & (np.abs(cen[:, d]) < 1e-12)
        sides[name + "1"] = bnd & (np.abs(cen[:, d] - 1.0) < 1e-12)
    return bnd, sides


def heat2d(N: int = 128, steps: int = 100, dt: float = 1e-4, tol: float = 1e-12, seed: int = 1234,
           form: int = L.FORM_FP64) -> Problem:
    coords, cells = meshgen.square_triangles(N, 0.2, seed)
    cen = meshgen.cell_centroids(coords, cells)
    Z0 = np.exp(-50.0 * ((cen - 0.5) ** 2).sum(axis=1))
    coeffs = {"N": 1.0, "u": 0.0, "m": 1.0, "D": 1.0, "w": 0.0, "a": 0.0, "r": 0.0, "f": 0.0, "m_upw": 1.0,
              "m_bnd": 1.0}

    def bc_fn(face_verts, face_cells):
        F = face_cells.shape[0]
        return (np.zeros(F, np.uint8), np.zeros(F), np.zeros(F))

    cfg = StaticConfig(dim=2, n_eq=1, mass_lumping=False, advection=L.EXPLICIT_UPWIND, mobility_upwind=False,
                       form=form)
    return Problem("heat2d", cfg, coords, cells, coeffs, Z0, dt, steps, tol, bc_fn, N)


def _diffusion_bc(coords):
    def bc_fn(face_verts, face_cells):
        F = face_cells.shape[0]
        bnd, sides = _boundary_sides(coords, face_verts, face_cells, 3)
        tags = np.zeros(F, np.uint8)
        tags[bnd] = BC_FIXED_FLUX
        tags[sides["x0"] | sides["x1"]] = BC_FIXED_VALUE
        return tags, np.zeros(F), np.zeros(F)
    return bc_fn


def diffusion3d(N: int = 64, steps: int = 50, dt: float = 1e-3, tol: float = 1e-10, seed: int = 1234,
                field_seed: int = 5678, form: int = L.FORM_FP64) -> Problem:
    coords, cells = meshgen.cube_tetrahedra(N, 0.15, seed)
    g = meshgen.gaussian_field((N, N, N), 0.1, field_seed)  # indexed [x][y][z]
    cen = meshgen.cell_centroids(coords, cells)
    gx, gy, gz = meshgen.cell_grid_index(cen, N)
    D = np.exp(g[gx, gy, gz])
    coeffs = {"N": 1.0, "u": 0.0, "m": 1.0, "D": D, "w": 0.0, "a": 0.0, "r": 0.0, "f": 1.0, "m_upw": 1.0,
              "m_bnd": 1.0}
    cfg = StaticConfig(dim=3, n_eq=1, mass_lumping=False, advection=L.EXPLICIT_UPWIND, mobility_upwind=False,
                       form=form)
    return Problem("diffusion3d", cfg, coords, cells, coeffs, np.zeros(cells.shape[0]), dt, steps, tol,
                   _diffusion_bc(coords), N)


def heat2d_rect(N: int = 128, steps: int = 100, dt: float = 1e-4, tol: float = 1e-12, lumping: bool = False,
                form: int = L.FORM_FP64) -> Problem:
    """The heat-equation workload on N x N graded rectangles (box cells)."""
    coords, cells = meshgen.square_rectangles(N)
    cen = meshgen.cell_centroids(coords, cells)
    Z0 = np.exp(-50.0 * ((cen - 0.5) ** 2).sum(axis=1))
    coeffs = {"N": 1.0, "u": 0.0, "m": 1.0, "D": 1.0, "w": 0.0, "a": 0.0, "r": 0.0, "f": 0.0, "m_upw": 1.0,
              "m_bnd": 1.0}

    def bc_fn(face_verts, face_cells):
        F = face_cells.shape[0]
        return (np.zeros(F, np.uint8), np.zeros(F), np.zeros(F))

    cfg = StaticConfig(dim=2, n_eq=1, mass_lumping=lumping, advection=L.EXPLICIT_UPWIND, mobility_upwind=False,
                       form=form, cell=L.CELL_BOX)
    return Problem("heat2d_rect", cfg, coords, cells, coeffs, Z0, dt, steps, tol, bc_fn, N)


def diffusion3d_box(N: int = 64, steps: int = 50, dt: float = 1e-3, tol: float = 1e-10, lumping: bool = False,
                    field_seed: int = 5678, form: int = L.FORM_FP64) -> Problem:
    """The heterogeneous-diffusion workload on N^3 graded cuboids (box cells)."""
    coords, cells = meshgen.cube_cuboids(N)
    g = meshgen.gaussian_field((N, N, N), 0.1, field_seed)
    cen = meshgen.cell_centroids(coords, cells)
    gx, gy, gz = meshgen.cell_grid_index(cen, N)
    D = np.exp(g[gx, gy, gz])
    coeffs = {"N": 1.0, "u": 0.0, "m": 1.0, "D": D, "w": 0.0, "a": 0.0, "r": 0.0, "f": 1.0, "m_upw": 1.0,
              "m_bnd": 1.0}
    cfg = StaticConfig(dim=3, n_eq=1, mass_lumping=lumping, advection=L.EXPLICIT_UPWIND, mobility_upwind=False,
                       form=form, cell=L.CELL_BOX)
    return Problem("diffusion3d_box", cfg, coords, cells, coeffs, np.zeros(cells.shape[0]), dt, steps, tol,
                   _diffusion_bc(coords), N)


def diffusion3d_source(N: int = 64, steps: int = 1000, dt: float = 1e-3, tol: float = 1e-10, seed: int = 1234,
                       field_seed: int = 5678, psi_seed: int = 9101, form: int = L.FORM_FP64) -> Problem:
    p = diffusion3d(N, steps, dt, tol, seed, field_seed, form)
    psi_grid = meshgen.gaussian_field((N, N, N), 0.2, psi_seed)
    cen = meshgen.cell_centroids(p.coords, p.cells)
    gx, gy, gz = meshgen.cell_grid_index(cen, N)
    p.coeffs["psi"] = psi_grid[gx, gy, gz]
    p.source = (0.5, steps * dt)
    p.name = "diffusion3d_source"
    return p


def adr2d(N: int = 512, steps: int = 200, dt: float = 5e-4, tol: float = 1e-10, seed: int = 1234,
          field_seed: int = 5678, form: int = L.FORM_FP64, box: bool = False) -> Problem:
    """box=True: the same model on N x N graded rectangles."""
    n = 2
    coords, cells = meshgen.square_rectangles(N) if box else meshgen.square_triangles(N, 0.2, seed)
    C = cells.shape[0]
    nf = 4 if box else 3
    g = meshgen.gaussian_field((N, N), 0.1, field_seed)
    cen = meshgen.cell_centroids(coords, cells)
    gx, gy = meshgen.cell_grid_index(cen, N)
    scale = np.exp(0.5 * g[gx, gy])
    Nc = np.zeros((n, n, C)); Nc[0, 0] = 1.0; Nc[1, 1] = 1.0
    D = np.zeros((n, n, C)); D[0, 0] = 1e-2 * scale; D[1, 1] = 5e-3 * scale
    r = np.zeros((n, n, C)); r[0, 0] = 0.1; r[0, 1] = -0.05; r[1, 0] = -0.05; r[1, 1] = 0.1
    # RT0 face fluxes of the constant advection field (1, 0.3): a_iiKe = a . n_Ke |E_e|
    normals = meshgen.outward_face_normals(coords, cells)  # [C][nf][2], scaled by |E|
    vel = np.array([1.0, 0.3])
    flux = np.einsum("cfd,d->fc", normals, vel)  # [e][K]
    a = np.zeros((n, n, nf, C)); a[0, 0] = flux; a[1, 1] = flux
    coeffs = {"N": Nc.ravel(), "u": 0.0, "m": 1.0, "D": D.ravel(), "w": 0.0, "a": a.ravel(), "r": r.ravel(),
              "f": 0.0, "m_upw": 1.0, "m_bnd": 1.0}

    def bc_fn(face_verts, face_cells):
        F = face_cells.shape[0]
        bnd, sides = _boundary_sides(coords, face_verts, face_cells, 2)
        tags = np.zeros((n, F), np.uint8)
        dirichlet = np.zeros((n, F))
        tags[:, bnd] = BC_FIXED_FLUX  # zero total flux on the walls y=0, y=1
        tags[:, sides["x1"]] = BC_ADVECTIVE_OUTFLOW
        tags[:, sides["x0"]] = BC_FIXED_VALUE
        dirichlet[0, sides["x0"]] = 1.0
        return tags.ravel(), np.zeros(n * F), dirichlet.ravel()

    cfg = StaticConfig(dim=2, n_eq=2, mass_lumping=True, advection=L.EXPLICIT_UPWIND, mobility_upwind=False,
                       form=form, cell=L.CELL_BOX if box else L.CELL_SIMPLEX)
    return Problem("adr2d_rect" if box else "adr2d", cfg, coords, cells, coeffs, np.zeros(n * C), dt, steps, tol,
                   bc_fn, N)


WORKLOADS = {
    "heat2d": heat2d,
    "diffusion3d": diffusion3d,
    "adr2d": adr2d,
    "diffusion3d_source": diffusion3d_source,
    "heat2d_rect": heat2d_rect,
    "diffusion3d_box": diffusion3d_box,
}


def make_solver(p: Problem, check_every: int = 8, max_iter: int = 20000, inner_tol: float = 1e-4):
    """Creates a Solver for the problem: mesh, coefficients, BCs, IC, pattern."""
    from .solver import Solver
    s = Solver(p.config)
    s.setMesh(p.coords, p.cells)
    for k, v in p.coeffs.items():
        s.set_coeff(k, v)
    if p.source is not None:
        s.set_source_modulation(*p.source)
    fv, fc, _ = s.topology()
    s.set_bc(*p.bc_fn(fv, fc))
    s.setup(tol=p.tol, max_iter=max_iter, inner_tol=inner_tol, check_every=check_every)
    s.setInitialCondition(p.Z0)
    s.setupLinearSystem()
    return s
