"""ctypes driver of the CPU oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module.  It runs the C restatement of the reference
algorithm (oracle/mhfem_oracle.c) on the same model definitions the product
path receives.  Parity status: unpinned (see mhfem_oracle.h).
"""
from __future__ import annotations

import ctypes as ct
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
LIB_PATH = ORACLE_DIR / "liboracle_mhfem.so"


class Coef(ct.Structure):
    _fields_ = [("p", ct.POINTER(ct.c_double)), ("full", ct.c_int)]


_pd = ct.POINTER(ct.c_double)
_pi32 = ct.POINTER(ct.c_int32)
_pi64 = ct.POINTER(ct.c_int64)
_pu8 = ct.POINTER(ct.c_uint8)


class OrcProblem(ct.Structure):
    _fields_ = [
        ("dim", ct.c_int), ("cell", ct.c_int), ("nf", ct.c_int), ("nv", ct.c_int), ("fv", ct.c_int),
        ("n", ct.c_int), ("S", ct.c_int), ("lumping", ct.c_int),
        ("advection", ct.c_int), ("mobility_upwind", ct.c_int),
        ("V", ct.c_int64), ("C", ct.c_int64), ("F", ct.c_int64),
        ("coords", _pd), ("cell_verts", _pi32), ("cell_faces", _pi32), ("face_cells", _pi32),
        ("N", Coef), ("u", Coef), ("m", Coef), ("D", Coef), ("w", Coef), ("a", Coef), ("r", Coef), ("f", Coef),
        ("m_bnd", Coef),
        ("bc_tags", _pu8), ("bc_values", _pd), ("bc_dirichlet", _pd),
        ("Z_iF", _pd), ("Z_iK", _pd), ("v_iKe", _pd), ("m_upw", _pd), ("m_upw_full", ct.c_int), ("Z_upw", _pd),
        ("b", _pd), ("R_ijKe", _pd), ("R_iK", _pd),
    ]


_lib = None


def load():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} missing: build it with tnl-mhfem_gb300/build.py")
        lib = ct.CDLL(str(LIB_PATH))
        lib.orc_build_faces_ct.restype = ct.c_int64
        lib.orc_build_faces_ct.argtypes = [ct.c_int, ct.c_int, ct.c_int64, _pi32, _pi32, _pi32, _pi32]
        for name in ["orc_face_average", "orc_update_b", "orc_reconstruct", "orc_velocities"]:
            getattr(lib, name).argtypes = [ct.POINTER(OrcProblem)]
            getattr(lib, name).restype = None
        lib.orc_upwind.argtypes = [ct.POINTER(OrcProblem), ct.c_double, ct.c_double]
        lib.orc_update_R.argtypes = [ct.POINTER(OrcProblem), ct.c_double]
        lib.orc_update_Q.argtypes = [ct.POINTER(OrcProblem), ct.c_double]
        lib.orc_row_lengths.argtypes = [ct.POINTER(OrcProblem), _pi32]
        lib.orc_assemble.restype = ct.c_int
        lib.orc_assemble.argtypes = [ct.POINTER(OrcProblem), _pi32, ct.c_double, ct.c_double, _pi64, _pi32, _pd, _pd]
        lib.orc_bicgstab.restype = ct.c_int
        lib.orc_bicgstab.argtypes = [ct.c_int64, _pi64, _pi32, _pd, _pd, _pd, ct.c_double, ct.c_int,
                                     ct.POINTER(ct.c_int), ct.POINTER(ct.c_double)]
        lib.orc_step.restype = ct.c_int
        lib.orc_step.argtypes = [ct.POINTER(OrcProblem), _pi32, ct.c_double, ct.c_double, _pi64, _pi32, _pd, _pd,
                                 ct.c_double, ct.c_int, ct.POINTER(ct.c_int), ct.POINTER(ct.c_double)]
        lib.orc_set_threads.argtypes = [ct.c_int]
        lib.orc_get_threads.restype = ct.c_int
        _lib = lib
    return _lib


def cell_shape(dim: int, cell: int = 0):
    """(faces per cell, vertices per cell, vertices per face, MassMatrix::size)."""
    if cell:
        return 2 * dim, 2 ** dim, 2 ** (dim - 1), dim
    return dim + 1, dim + 1, dim, 9 if dim == 2 else 14


def build_faces(dim: int, cells: np.ndarray, cell: int = 0):
    """Topology by the oracle's own (sort-based) builder."""
    lib = load()
    cells = np.ascontiguousarray(cells, np.int32)
    C = cells.shape[0]
    nf, _, nfv, _ = cell_shape(dim, cell)
    cf = np.empty((C, nf), np.int32)
    fc = np.empty((C * nf, 2), np.int32)
    fv = np.empty((C * nf, nfv), np.int32)
    F = lib.orc_build_faces_ct(dim, cell, C, cells.ctypes.data_as(_pi32), cf.ctypes.data_as(_pi32),
                               fc.ctypes.data_as(_pi32), fv.ctypes.data_as(_pi32))
    return fv[:F].copy(), fc[:F].copy(), cf


def _dp(a):
    return a.ctypes.data_as(_pd)


class OracleModel:
    """One MHFEM problem evaluated by the CPU oracle, mirroring the solver phases."""

    def __init__(self, dim, n, lumping, advection, mobility_upwind, coords, cells, coeffs, bc_fn, Z0,
                 threads: int = 0, cell: int = 0):
        self.lib = load()
        if threads:
            self.lib.orc_set_threads(threads)
        self.dim, self.n, self.cell = dim, n, int(cell)
        self.nf, self.nv, self.fv, self.S = cell_shape(dim, self.cell)
        self.coords = np.ascontiguousarray(coords, np.float64)
        self.cells = np.ascontiguousarray(cells, np.int32)
        self.face_verts, self.face_cells, self.cell_faces = build_faces(dim, self.cells, self.cell)
        self.C = self.cells.shape[0]
        self.F = self.face_cells.shape[0]
        self.V = self.coords.shape[0]
        C, F, nf, S = self.C, self.F, self.nf, self.S
        self._keep = []
        self.Z_iF = np.zeros(n * F)
        self.Z_iK = np.ascontiguousarray(np.asarray(Z0, np.float64).ravel().copy())
        self.v_iKe = np.zeros(n * nf * C)
        self.Z_upw = np.zeros(n * n * F)
        self.b = np.zeros(n * n * S * C)
        self.R_ijKe = np.zeros(n * n * nf * C)
        self.R_iK = np.zeros(n * C)
        tags, values, dirichlet = bc_fn(self.face_verts, self.face_cells)
        self.tags = np.ascontiguousarray(tags, np.uint8)
        self.bvalues = np.ascontiguousarray(values, np.float64)
        self.bdirichlet = np.ascontiguousarray(dirichlet, np.float64)
        P = OrcProblem()
        P.dim, P.cell, P.nf, P.nv, P.fv, P.n, P.S = dim, self.cell, nf, self.nv, self.fv, n, S
        P.lumping, P.advection, P.mobility_upwind = int(lumping), int(advection), int(mobility_upwind)
        P.V, P.C, P.F = self.V, C, F
        P.coords = _dp(self.coords)
        P.cell_verts = self.cells.ctypes.data_as(_pi32)
        P.cell_faces = self.cell_faces.ctypes.data_as(_pi32)
        P.face_cells = self.face_cells.ctypes.data_as(_pi32)
        # the coefficient arrays the restatement reads; a test may change their
        # values in place between steps (a model's updateNonLinearTerms)
        self.coeff_arrays = {}
        for name in ["N", "u", "m", "D", "w", "a", "r", "f", "m_bnd"]:
            arr = np.ascontiguousarray(np.atleast_1d(np.asarray(coeffs.get(name, 0.0), np.float64)).ravel())
            self._keep.append(arr)
            self.coeff_arrays[name] = arr
            setattr(P, name, Coef(_dp(arr), int(arr.size > 1)))
        m_upw = np.ascontiguousarray(np.atleast_1d(np.asarray(coeffs.get("m_upw", 1.0), np.float64)).ravel())
        if mobility_upwind:
            m_upw = np.zeros(n * F)
        self.m_upw = m_upw
        P.m_upw = _dp(self.m_upw)
        P.m_upw_full = int(m_upw.size > 1)
        P.bc_tags = self.tags.ctypes.data_as(_pu8)
        P.bc_values = _dp(self.bvalues)
        P.bc_dirichlet = _dp(self.bdirichlet)
        P.Z_iF, P.Z_iK, P.v_iKe, P.Z_upw = _dp(self.Z_iF), _dp(self.Z_iK), _dp(self.v_iKe), _dp(self.Z_upw)
        P.b, P.R_ijKe, P.R_iK = _dp(self.b), _dp(self.R_ijKe), _dp(self.R_iK)
        self.P = P
        # time-modulated source: f = f_base + amp sin(2 pi t / T) psi
        self.f_base = np.ascontiguousarray(np.atleast_1d(np.asarray(coeffs.get("f", 0.0), np.float64)).ravel())
        self.psi = coeffs.get("psi")
        self.source = None
        # a model's updateVectorCoefficients: called as vector_hook(model, t, tau)
        # after the b update and before upwinding (Solver.hpp:641-652); it may
        # change coeff_arrays in place (w, a, u, m_bnd)
        self.vector_hook = None
        # pattern
        rows = n * F
        rowlen = np.empty(rows, np.int32)
        self.lib.orc_row_lengths(ct.byref(P), rowlen.ctypes.data_as(_pi32))
        self.rowptr = np.zeros(rows + 1, np.int64)
        np.cumsum(rowlen, out=self.rowptr[1:])
        nnz = int(self.rowptr[-1])
        self.cols = np.zeros(nnz, np.int32)
        self.vals = np.zeros(nnz)
        self.rhs = np.zeros(rows)
        self.lib.orc_face_average(ct.byref(P))

    @classmethod
    def from_problem(cls, p, threads: int = 0):
        c = p.config
        m = cls(c.dim, c.n_eq, c.mass_lumping, c.advection, c.mobility_upwind, p.coords, p.cells, p.coeffs,
                p.bc_fn, p.Z0, threads, getattr(c, "cell", 0))
        if p.source is not None:
            m.set_source(*p.source)
        return m

    def set_source(self, amplitude: float, period: float):
        self.source = (amplitude, period)
        self._f_now = np.empty(self.n * self.C)
        self.P.f = Coef(_dp(self._f_now), 1)

    def _update_source(self, t: float):
        if self.source is None:
            return
        amp, period = self.source
        base = np.broadcast_to(self.f_base, (self.n * self.C,)) if self.f_base.size == 1 else self.f_base
        psi = np.tile(np.asarray(self.psi, np.float64), self.n)
        self._f_now[:] = base + amp * np.sin(2 * np.pi * t / period) * psi

    # phases -----------------------------------------------------------
    def pre_iterate(self, t, tau):
        self._update_source(t)
        P = ct.byref(self.P)
        self.lib.orc_update_b(P)
        if self.vector_hook is not None:
            self.vector_hook(self, t, tau)
        self.lib.orc_upwind(P, t, tau)
        self.lib.orc_update_R(P, tau)
        self.lib.orc_update_Q(P, tau)

    def assemble(self, t, tau):
        st = self.lib.orc_assemble(ct.byref(self.P), self.face_verts.ctypes.data_as(_pi32), t + tau, tau,
                                   self.rowptr.ctypes.data_as(_pi64), self.cols.ctypes.data_as(_pi32),
                                   _dp(self.vals), _dp(self.rhs))
        if st != 0:
            raise RuntimeError("oracle: non-positive diagonal")

    def solve(self, tol, max_iter=20000):
        it = ct.c_int()
        res = ct.c_double()
        st = self.lib.orc_bicgstab(self.n * self.F, self.rowptr.ctypes.data_as(_pi64),
                                   self.cols.ctypes.data_as(_pi32), _dp(self.vals), _dp(self.rhs), _dp(self.Z_iF),
                                   tol, max_iter, ct.byref(it), ct.byref(res))
        if st != 0:
            raise RuntimeError(f"oracle BiCGStab failed with status {st} after {it.value} iterations")
        return it.value, res.value

    def post_iterate(self, t, tau):
        self.lib.orc_reconstruct(ct.byref(self.P))
        if self.P.mobility_upwind:
            self.lib.orc_velocities(ct.byref(self.P))

    def step(self, t, tau, tol, max_iter=20000):
        self.pre_iterate(t, tau)
        self.assemble(t, tau)
        it, res = self.solve(tol, max_iter)
        self.post_iterate(t, tau)
        return it, res

    def csr(self):
        import scipy.sparse as sp
        rows = self.n * self.F
        return sp.csr_matrix((self.vals, self.cols, self.rowptr), shape=(rows, rows))
