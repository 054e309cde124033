"""Host-side mirror of TNL::MHFEM::Solver over the C ABI.

Method names follow the reference's Solver interface (Solver.h:64-117):
``setMesh``, ``setup``, ``setInitialCondition``, ``setupLinearSystem``,
``preIterate``, ``assembleLinearSystem``, ``solveLinearSystem``,
``postIterate``; ``step`` runs the four phases of one time step as
MHFEM::solve does (control.h:83-98) and ``solve`` is that time loop.
Arrays are numpy arrays in the reference's CUDA layouts (BaseModel.h:18-125).
"""
from __future__ import annotations

import ctypes as ct
from dataclasses import dataclass

import numpy as np

from . import _lib as L


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(ct.POINTER(ct.c_double))


def _i32ptr(a: np.ndarray):
    return a.ctypes.data_as(ct.POINTER(ct.c_int32))


def _i64ptr(a: np.ndarray):
    return a.ctypes.data_as(ct.POINTER(ct.c_int64))


@dataclass
class StaticConfig:
    """The reference's compile-time configuration (examples/config.h), at run time."""
    dim: int = 2
    n_eq: int = 1
    mass_lumping: bool = False
    advection: int = L.EXPLICIT_UPWIND
    mobility_upwind: bool = False
    form: int = L.FORM_FP64
    device: int = 0
    cell: int = L.CELL_SIMPLEX  # CELL_BOX: rectangles / cuboids

    @property
    def faces_per_cell(self) -> int:
        return 2 * self.dim if self.cell == L.CELL_BOX else self.dim + 1

    @property
    def verts_per_cell(self) -> int:
        return 2 ** self.dim if self.cell == L.CELL_BOX else self.dim + 1

    @property
    def verts_per_face(self) -> int:
        return 2 ** (self.dim - 1) if self.cell == L.CELL_BOX else self.dim


COEF_IDS = {"N": L.COEF_N, "u": L.COEF_U, "m": L.COEF_M, "D": L.COEF_D, "w": L.COEF_W, "a": L.COEF_A,
            "r": L.COEF_R, "f": L.COEF_F, "m_upw": L.COEF_M_UPW, "m_bnd": L.COEF_M_BND, "psi": L.COEF_PSI}
ARRAY_IDS = {"b": L.ARRAY_B, "R_ijKe": L.ARRAY_R_IJKE, "R_iK": L.ARRAY_R_IK, "m_upw": L.ARRAY_M_UPW,
             "Z_upw": L.ARRAY_Z_UPW, "v_iKe": L.ARRAY_V, "rhs": L.ARRAY_RHS, "Z_iF": L.ARRAY_Z_IF,
             "Z_iK": L.ARRAY_Z_IK}


class DeviceArray:
    """A library-owned FP64 device array, exposed through
    ``__cuda_array_interface__`` (so ``torch.as_tensor(a, device="cuda")``
    or any CUDA array library views it without a copy)."""

    def __init__(self, ptr: int, count: int):
        self.ptr, self.count = ptr, count

    @property
    def __cuda_array_interface__(self):
        return {"shape": (self.count,), "typestr": "<f8", "data": (self.ptr, False), "version": 2,
                "strides": None}


class Solver:
    def __init__(self, config: StaticConfig):
        self.lib = L.load()
        self.config = config
        desc = L.Desc(config.dim, config.n_eq, int(config.mass_lumping), config.advection,
                      int(config.mobility_upwind), config.form, config.device, config.cell)
        h = ct.c_void_p()
        st = self.lib.mhfem_create(ct.byref(desc), ct.byref(h))
        if st != L.OK:
            raise L.MhfemError(st, "mhfem_create failed (is a CUDA device visible?)")
        self._h = h
        self.C = self.F = self.V = 0
        self.time_steps = 0

    # -- error handling --------------------------------------------------
    def _ck(self, st: int) -> None:
        if st != L.OK:
            msg = self.lib.mhfem_last_error(self._h)
            raise L.MhfemError(st, msg.decode() if msg else "")

    def close(self) -> None:
        if getattr(self, "_h", None):
            self.lib.mhfem_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- setup (Solver.hpp:28-484) -----------------------------------------
    def setMesh(self, coords: np.ndarray, cells: np.ndarray) -> None:
        coords = np.ascontiguousarray(coords, dtype=np.float64)
        cells = np.ascontiguousarray(cells, dtype=np.int32)
        if coords.ndim != 2 or coords.shape[1] != self.config.dim:
            raise ValueError(f"coords must have shape (V, {self.config.dim}), got {coords.shape}")
        if cells.ndim != 2 or cells.shape[1] != self.config.verts_per_cell:
            raise ValueError(f"cells must have shape (C, {self.config.verts_per_cell}), got {cells.shape}")
        self._ck(self.lib.mhfem_set_mesh(self._h, coords.shape[0], _dptr(coords), cells.shape[0], _i32ptr(cells)))
        V = ct.c_int64(); C = ct.c_int64(); F = ct.c_int64()
        self._ck(self.lib.mhfem_get_sizes(self._h, ct.byref(V), ct.byref(C), ct.byref(F), None, None))
        self.V, self.C, self.F = V.value, C.value, F.value

    def topology(self):
        fv = np.empty((self.F, self.config.verts_per_face), np.int32)
        fc = np.empty((self.F, 2), np.int32)
        cf = np.empty((self.C, self.config.faces_per_cell), np.int32)
        self._ck(self.lib.mhfem_get_topology(self._h, _i32ptr(fv), _i32ptr(fc), _i32ptr(cf)))
        return fv, fc, cf

    def set_coeff(self, name: str, value) -> None:
        arr = np.ascontiguousarray(np.atleast_1d(np.asarray(value, dtype=np.float64)).ravel())
        self._ck(self.lib.mhfem_set_coeff(self._h, COEF_IDS[name], _dptr(arr), arr.size))

    def set_source_modulation(self, amplitude: float, period: float) -> None:
        self._ck(self.lib.mhfem_set_source_modulation(self._h, amplitude, period))

    def set_bc(self, tags: np.ndarray, values: np.ndarray, dirichlet: np.ndarray) -> None:
        tags = np.ascontiguousarray(tags, dtype=np.uint8)
        values = np.ascontiguousarray(values, dtype=np.float64)
        dirichlet = np.ascontiguousarray(dirichlet, dtype=np.float64)
        n = self.config.n_eq * self.F
        if tags.size != n or values.size != n or dirichlet.size != n:
            raise ValueError(f"boundary arrays must hold n*F = {n} entries")
        self._ck(self.lib.mhfem_set_bc(self._h, tags.ctypes.data_as(ct.POINTER(ct.c_uint8)), _dptr(values),
                                       _dptr(dirichlet)))

    def setup(self, tol: float = 1e-10, max_iter: int = 10000, inner_tol: float = 1e-4, max_sweeps: int = 50,
              check_every: int = 8, timeout_s: float = 0.0, inner_adaptive: bool = True,
              linear_solver: str = "bicgstab", gmres_restart: int = 30, gmres_variant: str = "cgs",
              gmres_restart_min: int = 0, gmres_restart_step_min: int = 0, gmres_restart_step_max: int = 0) -> None:
        """Solver::setup (Solver.hpp:88-258): the Krylov solver ("bicgstab" or
        "gmres" with restart length gmres_restart and variant "cgs" / "cgsr";
        with gmres_restart_min and the steps set, the restart length varies
        between gmres_restart_min and gmres_restart), its tolerance and caps,
        and the mixed form's inner-solve options."""
        solvers = {"bicgstab": L.SOLVER_BICGSTAB, "gmres": L.SOLVER_GMRES}
        variants = {"cgs": L.GMRES_CGS, "cgsr": L.GMRES_CGSR}
        o = L.SolverOpts(tol, max_iter, inner_tol, max_sweeps, check_every, timeout_s, int(inner_adaptive),
                         solvers[linear_solver.lower()], gmres_restart, variants[gmres_variant.lower()],
                         gmres_restart_min, gmres_restart_step_min, gmres_restart_step_max)
        self._ck(self.lib.mhfem_set_solver(self._h, ct.byref(o)))

    def setInitialCondition(self, Z_iK: np.ndarray, Z_iF: np.ndarray | None = None) -> None:
        n = self.config.n_eq
        Z_iK = np.ascontiguousarray(Z_iK, dtype=np.float64).ravel()
        if Z_iK.size != n * self.C:
            raise ValueError(f"Z_iK must hold n*C = {n * self.C} values, got {Z_iK.size}")
        if Z_iF is None:
            self._ck(self.lib.mhfem_set_initial_condition(self._h, _dptr(Z_iK)))
        else:
            Z_iF = np.ascontiguousarray(Z_iF, dtype=np.float64).ravel()
            if Z_iF.size != n * self.F:
                raise ValueError(f"Z_iF must hold n*F = {n * self.F} values, got {Z_iF.size}")
            self._ck(self.lib.mhfem_set_state(self._h, _dptr(Z_iK), _dptr(Z_iF)))

    def setupLinearSystem(self) -> None:
        self._ck(self.lib.mhfem_setup_linear_system(self._h))

    # -- one time step (control.h:83-98) -------------------------------
    def preIterate(self, t: float, tau: float) -> None:
        self._ck(self.lib.mhfem_pre_iterate(self._h, t, tau))

    def assembleLinearSystem(self, t: float, tau: float) -> None:
        self._ck(self.lib.mhfem_assemble(self._h, t, tau))

    def solveLinearSystem(self) -> dict:
        s = L.StepStats()
        self._ck(self.lib.mhfem_solve(self._h, ct.byref(s)))
        return s.as_dict()

    def postIterate(self, t: float, tau: float) -> None:
        self._ck(self.lib.mhfem_post_iterate(self._h, t, tau))

    def step(self, t: float, tau: float, stats: bool = True) -> dict | None:
        if stats:
            s = L.StepStats()
            self._ck(self.lib.mhfem_step(self._h, t, tau, ct.byref(s)))
            self.time_steps += 1
            return s.as_dict()
        self._ck(self.lib.mhfem_step(self._h, t, tau, None))
        self.time_steps += 1
        return None

    def solve(self, start_time: float, stop_time: float, time_step: float, callback=None) -> list:
        """The time loop of MHFEM::solve (control.h:64-102)."""
        t = start_time
        out = []
        while stop_time - t > time_step * 1e-6:
            tau = min(time_step, stop_time - t)
            st = self.step(t, tau)
            out.append(st)
            if callback:
                callback(t, tau, st)
            t += tau
        return out

    # -- results --------------------------------------------------------
    def state(self):
        zf = np.empty(self.config.n_eq * self.F)
        zk = np.empty(self.config.n_eq * self.C)
        self._ck(self.lib.mhfem_get_state(self._h, _dptr(zf), _dptr(zk)))
        return zf, zk

    def array(self, name: str, size: int) -> np.ndarray:
        out = np.empty(size)
        self._ck(self.lib.mhfem_get_array(self._h, ARRAY_IDS[name], _dptr(out), size))
        return out

    def system(self):
        rows = ct.c_int64(); nnz = ct.c_int64()
        self._ck(self.lib.mhfem_get_sizes(self._h, None, None, None, ct.byref(rows), ct.byref(nnz)))
        rowptr = np.empty(rows.value + 1, np.int64)
        cols = np.empty(nnz.value, np.int32)
        vals = np.empty(nnz.value)
        rhs = np.empty(rows.value)
        self._ck(self.lib.mhfem_get_system(self._h, _i64ptr(rowptr), _i32ptr(cols), _dptr(vals), _dptr(rhs)))
        return rowptr, cols, vals, rhs

    def system32(self) -> np.ndarray:
        """The FP32 copy of the matrix values (mixed form), CSR order of system()."""
        nnz = ct.c_int64()
        self._ck(self.lib.mhfem_get_sizes(self._h, None, None, None, None, ct.byref(nnz)))
        out = np.empty(nnz.value, np.float32)
        self._ck(self.lib.mhfem_get_system32(self._h, out.ctypes.data_as(ct.POINTER(ct.c_float))))
        return out

    def totals(self):
        """(Krylov iterations, time steps, kernel launches) since creation."""
        it = ct.c_int64(); ts = ct.c_int64(); kl = ct.c_int64()
        self._ck(self.lib.mhfem_get_totals(self._h, ct.byref(it), ct.byref(ts), ct.byref(kl)))
        return it.value, ts.value, kl.value

    def set_hook(self, point: int, fn) -> None:
        """Model hook: fn(t, tau, stream) is called at `point` with the
        library's stream, on which its device work must be ordered.
        HOOK_PRE_ITERATE (updateNonLinearTerms): before this step's b update;
        HOOK_VECTOR_COEFFICIENTS (updateVectorCoefficients): after the b
        update, before upwinding, so u, w, a projections may read this step's
        b (and a model rewrites its boundary mobility m_bnd here);
        HOOK_POST_ITERATE: after the reconstruction.  None removes it."""
        if not hasattr(self, "_hooks"):
            self._hooks = {}
        if fn is None:
            cb = ct.cast(None, L.HOOK)
        else:
            cb = L.HOOK(lambda user, t, tau, stream: fn(t, tau, stream or 0))
        self._hooks[point] = cb  # keep the callback alive as long as the solver
        self._ck(self.lib.mhfem_set_hook(self._h, point, cb, None))

    def coeff_device(self, name: str) -> DeviceArray:
        """The device storage of a coefficient (size 1 when uniform)."""
        p = ct.c_void_p(); n = ct.c_int64()
        self._ck(self.lib.mhfem_coeff_device(self._h, COEF_IDS[name], ct.byref(p), ct.byref(n)))
        return DeviceArray(p.value, n.value)

    def array_device(self, name: str) -> DeviceArray:
        """The device storage of a scheme / state array (b, R_ijKe, R_iK, m_upw, Z_upw, v_iKe, rhs, Z_iF, Z_iK)."""
        p = ct.c_void_p(); n = ct.c_int64()
        self._ck(self.lib.mhfem_array_device(self._h, ARRAY_IDS[name], ct.byref(p), ct.byref(n)))
        return DeviceArray(p.value, n.value)

    def stream(self) -> int:
        """The library's CUDA stream handle (for CUDA events on that stream)."""
        p = ct.c_void_p()
        self._ck(self.lib.mhfem_get_stream(self._h, ct.byref(p)))
        return p.value or 0

    def time_kernel(self, kernel: int, reps: int = 20) -> dict:
        """Mean CUDA-event time of one path kernel and its algorithmic bytes / FLOPs per launch."""
        ms = ct.c_double(); b = ct.c_double(); fl = ct.c_double()
        self._ck(self.lib.mhfem_time_kernel(self._h, kernel, reps, ct.byref(ms), ct.byref(b), ct.byref(fl)))
        return {"ms": ms.value, "bytes": b.value, "flops": fl.value}

    # -- learned warm start (MHFEM_FORM_LEARNED) ------------------------
    def learned_options(self, train_steps: int = 200, train_iters: int = 2, learning_rate: float = 1e-3,
                        use_during_training: bool = False, seed: int = 0, lr_final: float = 1.0,
                        mixed_solve: bool = False, extrapolation_order: int = 3) -> None:
        o = L.LearnedOpts(train_steps, train_iters, learning_rate, int(use_during_training), seed, lr_final,
                          int(mixed_solve), extrapolation_order)
        self._ck(self.lib.mhfem_learned_set_options(self._h, ct.byref(o)))

    def learned_num_params(self) -> int:
        n = ct.c_int32()
        self._ck(self.lib.mhfem_learned_status(self._h, None, None, ct.byref(n)))
        return n.value

    def learned_params(self) -> np.ndarray:
        out = np.empty(self.learned_num_params(), np.float32)
        self._ck(self.lib.mhfem_learned_get_params(self._h, out.ctypes.data_as(ct.POINTER(ct.c_float)), out.size))
        return out

    def set_learned_params(self, params: np.ndarray) -> None:
        p = np.ascontiguousarray(params, np.float32)
        self._ck(self.lib.mhfem_learned_set_params(self._h, p.ctypes.data_as(ct.POINTER(ct.c_float)), p.size))

    def _features(self, features: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(features, np.float32)
        if x.shape != (self.F, L.LEARNED_FEATURES):
            raise ValueError(f"features must have shape ({self.F}, {L.LEARNED_FEATURES}), got {x.shape}")
        return x

    def learned_forward(self, features: np.ndarray) -> np.ndarray:
        x = self._features(features)
        out = np.empty(self.F, np.float32)
        self._ck(self.lib.mhfem_learned_forward(self._h, x.ctypes.data_as(ct.POINTER(ct.c_float)),
                                                out.ctypes.data_as(ct.POINTER(ct.c_float))))
        return out

    def learned_gradients(self, features: np.ndarray, target: np.ndarray):
        x = self._features(features)
        y = np.ascontiguousarray(target, np.float64)
        if y.shape != (self.F,):
            raise ValueError(f"target must have shape ({self.F},), got {y.shape}")
        g = np.empty(self.learned_num_params(), np.float32)
        loss = ct.c_double()
        self._ck(self.lib.mhfem_learned_gradients(self._h, x.ctypes.data_as(ct.POINTER(ct.c_float)), _dptr(y),
                                                  g.ctypes.data_as(ct.POINTER(ct.c_float)), ct.byref(loss)))
        return loss.value, g

    def learned_status(self):
        ts = ct.c_int32(); ll = ct.c_double(); n = ct.c_int32()
        self._ck(self.lib.mhfem_learned_status(self._h, ct.byref(ts), ct.byref(ll), ct.byref(n)))
        return {"trained_steps": ts.value, "last_loss": ll.value, "num_params": n.value}
