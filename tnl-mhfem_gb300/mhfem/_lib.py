"""ctypes binding of the C ABI declared in include/mhfem.h.

The CUDA library is the only implementation: when ``libmhfem_gb300.so`` is
missing or no CUDA device is visible, loading raises instead of falling back
to anything else.
"""
from __future__ import annotations

import ctypes as ct
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent
LIB_PATH = PKG_ROOT / "libmhfem_gb300.so"

# status codes
OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_STATE = 2
ERR_CUDA = 3
ERR_NOT_CONVERGED = 4
ERR_BREAKDOWN = 5
ERR_NONPOSITIVE_DIAGONAL = 6
ERR_NO_DEVICE = 7
ERR_OUT_OF_MEMORY = 8
ERR_NOT_FINITE = 9
ERR_TIMEOUT = 10
ERR_UNSUPPORTED = 11

STATUS_NAMES = {
    0: "MHFEM_OK", 1: "MHFEM_ERR_INVALID_ARGUMENT", 2: "MHFEM_ERR_STATE", 3: "MHFEM_ERR_CUDA",
    4: "MHFEM_ERR_NOT_CONVERGED", 5: "MHFEM_ERR_BREAKDOWN", 6: "MHFEM_ERR_NONPOSITIVE_DIAGONAL",
    7: "MHFEM_ERR_NO_DEVICE", 8: "MHFEM_ERR_OUT_OF_MEMORY", 9: "MHFEM_ERR_NOT_FINITE",
    10: "MHFEM_ERR_TIMEOUT", 11: "MHFEM_ERR_UNSUPPORTED",
}

EXPLICIT_UPWIND, IMPLICIT_UPWIND, IMPLICIT_TRACE = 0, 1, 2
FORM_FP64, FORM_MIXED, FORM_LEARNED = 0, 1, 2

COEF_N, COEF_U, COEF_M, COEF_D, COEF_W, COEF_A, COEF_R, COEF_F, COEF_M_UPW, COEF_M_BND, COEF_PSI = range(11)
ARRAY_B, ARRAY_R_IJKE, ARRAY_R_IK, ARRAY_M_UPW, ARRAY_Z_UPW, ARRAY_V, ARRAY_RHS, ARRAY_Z_IF, ARRAY_Z_IK = range(9)
HOOK_PRE_ITERATE, HOOK_POST_ITERATE, HOOK_VECTOR_COEFFICIENTS = 0, 1, 2
# void hook(void* user, double t, double tau, void* stream)
HOOK = ct.CFUNCTYPE(None, ct.c_void_p, ct.c_double, ct.c_double, ct.c_void_p)
(KERNEL_CELL_LOCAL, KERNEL_ASSEMBLE, KERNEL_SPMV_FP64, KERNEL_SPMV_FP32, KERNEL_RECONSTRUCT, KERNEL_SPMV2_FP64,
 KERNEL_UPDATE_S_FP64, KERNEL_UPDATE_XR_FP64, KERNEL_UPDATE_P_FP64) = range(9)


class Desc(ct.Structure):
    _fields_ = [("dim", ct.c_int32), ("n_eq", ct.c_int32), ("mass_lumping", ct.c_int32),
                ("advection", ct.c_int32), ("mobility_upwind", ct.c_int32), ("form", ct.c_int32),
                ("device", ct.c_int32), ("cell", ct.c_int32)]


CELL_SIMPLEX = 0
CELL_BOX = 1


class SolverOpts(ct.Structure):
    _fields_ = [("tol", ct.c_double), ("max_iter", ct.c_int32), ("inner_tol", ct.c_double),
                ("max_sweeps", ct.c_int32), ("check_every", ct.c_int32), ("timeout_s", ct.c_double),
                ("inner_adaptive", ct.c_int32), ("linear_solver", ct.c_int32), ("gmres_restart", ct.c_int32),
                ("gmres_variant", ct.c_int32), ("gmres_restart_min", ct.c_int32),
                ("gmres_restart_step_min", ct.c_int32), ("gmres_restart_step_max", ct.c_int32)]


SOLVER_BICGSTAB, SOLVER_GMRES = 0, 1
GMRES_CGS, GMRES_CGSR = 0, 1


class LearnedOpts(ct.Structure):
    _fields_ = [("train_steps", ct.c_int32), ("train_iters", ct.c_int32), ("learning_rate", ct.c_double),
                ("use_during_training", ct.c_int32), ("seed", ct.c_uint64), ("lr_final", ct.c_double),
                ("mixed_solve", ct.c_int32), ("extrapolation_order", ct.c_int32)]


LEARNED_FEATURES = 16


class StepStats(ct.Structure):
    _fields_ = [("iterations", ct.c_int32), ("sweeps", ct.c_int32), ("residual", ct.c_double),
                ("guess_used", ct.c_int32), ("guess_residual", ct.c_double), ("warm_residual", ct.c_double),
                ("ms_pre", ct.c_double), ("ms_assemble", ct.c_double), ("ms_solve", ct.c_double),
                ("ms_post", ct.c_double), ("ms_guess", ct.c_double), ("base_residual", ct.c_double),
                ("guess_source", ct.c_int32)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


# Every exported symbol with its signature: (name, restype, argtypes).
_P = ct.c_void_p
_pd = ct.POINTER(ct.c_double)
_pi32 = ct.POINTER(ct.c_int32)
_pi64 = ct.POINTER(ct.c_int64)
_pu8 = ct.POINTER(ct.c_uint8)
SIGNATURES = [
    ("mhfem_create", ct.c_int32, [ct.POINTER(Desc), ct.POINTER(_P)]),
    ("mhfem_destroy", ct.c_int32, [_P]),
    ("mhfem_last_error", ct.c_char_p, [_P]),
    ("mhfem_default_solver_opts", None, [ct.POINTER(SolverOpts)]),
    ("mhfem_set_mesh", ct.c_int32, [_P, ct.c_int64, _pd, ct.c_int64, _pi32]),
    ("mhfem_get_sizes", ct.c_int32, [_P, _pi64, _pi64, _pi64, _pi64, _pi64]),
    ("mhfem_get_topology", ct.c_int32, [_P, _pi32, _pi32, _pi32]),
    ("mhfem_set_coeff", ct.c_int32, [_P, ct.c_int32, _pd, ct.c_int64]),
    ("mhfem_set_source_modulation", ct.c_int32, [_P, ct.c_double, ct.c_double]),
    ("mhfem_set_hook", ct.c_int32, [_P, ct.c_int32, HOOK, _P]),
    ("mhfem_coeff_device", ct.c_int32, [_P, ct.c_int32, ct.POINTER(_P), _pi64]),
    ("mhfem_array_device", ct.c_int32, [_P, ct.c_int32, ct.POINTER(_P), _pi64]),
    ("mhfem_set_bc", ct.c_int32, [_P, _pu8, _pd, _pd]),
    ("mhfem_set_initial_condition", ct.c_int32, [_P, _pd]),
    ("mhfem_set_state", ct.c_int32, [_P, _pd, _pd]),
    ("mhfem_set_solver", ct.c_int32, [_P, ct.POINTER(SolverOpts)]),
    ("mhfem_setup_linear_system", ct.c_int32, [_P]),
    ("mhfem_pre_iterate", ct.c_int32, [_P, ct.c_double, ct.c_double]),
    ("mhfem_assemble", ct.c_int32, [_P, ct.c_double, ct.c_double]),
    ("mhfem_solve", ct.c_int32, [_P, ct.POINTER(StepStats)]),
    ("mhfem_post_iterate", ct.c_int32, [_P, ct.c_double, ct.c_double]),
    ("mhfem_step", ct.c_int32, [_P, ct.c_double, ct.c_double, ct.POINTER(StepStats)]),
    ("mhfem_get_state", ct.c_int32, [_P, _pd, _pd]),
    ("mhfem_get_array", ct.c_int32, [_P, ct.c_int32, _pd, ct.c_int64]),
    ("mhfem_get_system", ct.c_int32, [_P, _pi64, _pi32, _pd, _pd]),
    ("mhfem_get_system32", ct.c_int32, [_P, ct.POINTER(ct.c_float)]),
    ("mhfem_get_totals", ct.c_int32, [_P, _pi64, _pi64, _pi64]),
    ("mhfem_get_stream", ct.c_int32, [_P, ct.POINTER(ct.c_void_p)]),
    ("mhfem_time_kernel", ct.c_int32, [_P, ct.c_int32, ct.c_int32, _pd, _pd, _pd]),
    ("mhfem_check_grid_barrier", ct.c_int32, [ct.c_int32, ct.c_int32, ct.c_int32, ct.c_int32, _pi32, _pi32, _pi32]),
    ("mhfem_learned_set_options", ct.c_int32, [_P, ct.POINTER(LearnedOpts)]),
    ("mhfem_learned_get_params", ct.c_int32, [_P, ct.POINTER(ct.c_float), ct.c_int64]),
    ("mhfem_learned_set_params", ct.c_int32, [_P, ct.POINTER(ct.c_float), ct.c_int64]),
    ("mhfem_learned_forward", ct.c_int32, [_P, ct.POINTER(ct.c_float), ct.POINTER(ct.c_float)]),
    ("mhfem_learned_gradients", ct.c_int32, [_P, ct.POINTER(ct.c_float), _pd, ct.POINTER(ct.c_float), _pd]),
    ("mhfem_learned_status", ct.c_int32, [_P, _pi32, _pd, _pi32]),
    ("mhfem_bicgstab_noalloc", ct.c_int32, [_P, _P, ct.c_int32, ct.c_int64, _P, _P, ct.c_double, ct.c_int32,
                                            ct.c_double, _pi32, _pd, _P]),
]
NOALLOC_MAX_ROWS = 262144

_lib = None


def load(path: Path | None = None) -> ct.CDLL:
    """Loads the CUDA library (no fallback: raises if it is missing)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build the CUDA library first (python __graft_entry__.py build "
            "or tnl-mhfem_gb300/build.py); the MHFEM solver has no CPU fallback")
    lib = ct.CDLL(str(p))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class MhfemError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status
