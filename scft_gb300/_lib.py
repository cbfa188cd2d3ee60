"""ctypes declarations of libscft.so (the C ABI in include/scft.h).

The library is built in-tree by ``scft_gb300.build`` (``__graft_entry__.build()``).
Loading fails loudly when it is missing: there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libscft.so")

SCFT_OK = 0
SCFT_EINVAL = -1
SCFT_ECUDA = -2
SCFT_ENOMEM = -3
SCFT_ENOCONFIG = -4
SCFT_ENODEV = -5
SCFT_ESINGULAR = -6
SCFT_EIO = -7

ST_NOT_DOMINANT = 1
ST_NONFINITE = 2
ST_CONVERGED = 4
ST_MAXIT = 8
ST_RESTARTED = 16
ST_WATCHDOG = 32
ST_FP64 = 64
ST_FORKED = 128
MAX_FORKS = 4

RULE_ROMBERG, RULE_TRAPEZOID = 0, 1
F32, F64 = 0, 1
SCHEME_IE, SCHEME_IRK2 = 0, 1
W_ROWSCALED, W_CONSISTENT = 0, 1
MIX_LINEAR, MIX_LOG = 0, 1

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)
VECFUNC = C.CFUNCTYPE(None, C.c_int, _dp, _dp)


class ScftConfig(C.Structure):
    _fields_ = [("n_nodes", C.c_int), ("x", _dp), ("L", C.c_double), ("f0", _dp),
                ("nsteps", C.c_int), ("ds", C.c_double), ("rule", C.c_int), ("sign", C.c_int),
                ("precision", C.c_int), ("scheme", C.c_int), ("wmode", C.c_int), ("w_wall", C.c_double * 2)]


class ScftInstance(C.Structure):
    _fields_ = [("n_nodes", C.c_int), ("x", _dp), ("L", C.c_double), ("f0", _dp), ("w0", _dp),
                ("nsteps", C.c_int), ("ds", C.c_double), ("rule", C.c_int)]


class ScftSolveOpts(C.Structure):
    _fields_ = [("precision", C.c_int), ("tol", C.c_double), ("tol32_factor", C.c_double),
                ("verify64", C.c_int), ("maxit", C.c_int), ("depth", C.c_int), ("beta", C.c_double),
                ("clip", C.c_double), ("grow", C.c_double), ("reg", C.c_double),
                ("residual_mode", C.c_int), ("precond", C.c_double), ("iters_per_graph", C.c_int),
                ("beta_schedule", C.c_int), ("weighted", C.c_int), ("step_cap", C.c_double),
                ("field_floor", C.c_double), ("fused", C.c_int),
                ("finish_stall", C.c_int), ("finish_tol", C.c_double), ("budget_ms", C.c_double),
                ("forks", C.c_int), ("fork_at", C.c_int), ("fork_grace", C.c_int), ("fork_first", C.c_int),
                ("fork_err", C.c_double),
                ("fork_scale", C.c_double * 4), ("graded_ratio", C.c_double), ("precond_hfloor", C.c_double),
                ("transfer_stride", C.c_int)]


class ScftResult(C.Structure):
    _fields_ = [("status", C.c_int), ("iterations", C.c_int), ("err", C.c_double), ("Q", C.c_double)]


# name -> (restype, argtypes); every function declared in include/scft.h
SIGNATURES = {
    "scft_config_init": (None, [C.POINTER(ScftConfig)]),
    "scft_set_config": (C.c_int, [C.POINTER(ScftConfig)]),
    "scft_fem_residual": (C.c_int, [C.c_int, _dp, _dp]),
    "scft_fem_residual_vf": (None, [C.c_int, _dp, _dp]),
    "scft_fem_residual0_vf": (None, [C.c_int, _dp, _dp]),
    "scft_fem_fixedpoint_vf": (None, [C.c_int, _dp, _dp]),
    "scft_density": (C.c_int, [_dp, _dp, _dp]),
    "scft_last_error": (C.c_char_p, []),
    "scft_strerror": (C.c_char_p, [C.c_int]),
    "scft_adm": (C.c_int, [_dp, C.c_int, C.POINTER(C.c_int), C.c_void_p, C.c_int]),
    "scft_adm_set_maxit": (None, [C.c_int]),
    "scft_adm_chen": (C.c_int, [C.c_void_p, _dp, C.c_double, C.c_int, C.c_int, C.c_double, C.c_int,
                                C.c_int]),
    "scft_broydn": (C.c_int, [_dp, C.c_int, C.POINTER(C.c_int), C.c_void_p]),
    "scft_nr_adm": (_dp, [_dp, C.c_int, C.POINTER(C.c_int), C.c_void_p, C.c_int]),
    "scft_nr_free_vector": (None, [_dp, C.c_int]),
    "scft_nr_broydn": (None, [_dp, C.c_int, C.POINTER(C.c_int), C.c_void_p]),
    "scft_broydn_set_tol": (None, [C.c_double]),
    "scft_broydn_get_err": (C.c_double, []),
    "scft_solve_opts_init": (None, [C.POINTER(ScftSolveOpts)]),
    "scft_batch_create": (C.c_int, [C.POINTER(ScftInstance), C.c_int, C.POINTER(C.c_void_p)]),
    "scft_batch_set_fields": (C.c_int, [C.c_void_p, _dp]),
    "scft_batch_evaluate": (C.c_int, [C.c_void_p, C.c_int]),
    "scft_batch_solve": (C.c_int, [C.c_void_p, C.POINTER(ScftSolveOpts), C.POINTER(ScftResult)]),
    "scft_batch_get": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
    "scft_batch_status": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "scft_batch_reset": (C.c_int, [C.c_void_p]),
    "scft_batch_last_ms": (C.c_double, [C.c_void_p]),
    "scft_batch_trace": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), _dp]),
    "scft_batch_free_energy": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp]),
    "scft_batch_live_stats": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _ip, _ip, C.POINTER(C.c_longlong), _dp, _dp]),
    "scft_batch_profile": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                     C.POINTER(C.c_int), _dp, _dp]),
    "scft_batch_set_shape": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]),
    "scft_batch_autotune": (C.c_int, [C.c_void_p, C.c_int]),
    "scft_batch_destroy": (C.c_int, [C.c_void_p]),
    "scft_kernel_launches": (C.c_longlong, []),
    "scft_mem_trim": (C.c_longlong, []),
    "scft_refine_bisect": (C.c_int, [C.c_int, _dp, _dp]),
    "scft_spline": (C.c_int, [C.c_int, C.POINTER(C.c_int), _dp, _dp, C.POINTER(C.c_int), _dp, _dp, _dp]),
    "scft_batch_solve_async": (C.c_int, [C.c_void_p, C.POINTER(ScftSolveOpts)]),
    "scft_batch_wait": (C.c_int, [C.c_void_p, C.POINTER(ScftResult)]),
    "scft_batch_evaluate_scheme": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "scft_ws_create": (C.c_int, [C.c_int, C.c_ulonglong, C.POINTER(C.c_void_p)]),
    "scft_ws_destroy": (C.c_int, [C.c_void_p]),
    "scft_ws_param_count": (C.c_int, [C.c_void_p]),
    "scft_ws_get_params": (C.c_int, [C.c_void_p, _fp]),
    "scft_ws_set_params": (C.c_int, [C.c_void_p, _fp]),
    "scft_ws_forward": (C.c_int, [C.c_void_p, _fp, C.c_int, _fp]),
    "scft_ws_loss_grad": (C.c_int, [C.c_void_p, _fp, _fp, C.c_int, _dp, _fp]),
    "scft_ws_batch_features": (C.c_int, [C.c_void_p, _fp, _fp]),
    "scft_ws_dataset_from_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_int)]),
    "scft_ws_train": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_ulonglong, _fp]),
    "scft_ws_predict": (C.c_int, [C.c_void_p, C.c_void_p]),
    "scft_ws_last_error": (C.c_char_p, []),
    "scft_ws_set_tensor_cores": (C.c_int, [C.c_void_p, C.c_int]),
    "scft_ws_tensor_core_status": (C.c_int, [C.c_void_p]),
    "scft_density_noalloc": (C.c_int, [C.c_int, _dp, _dp, C.c_int, C.c_double, C.c_int, C.c_int, _dp, _dp,
                                       C.POINTER(C.c_int), C.c_void_p]),
    "scft_mem_counters": (None, [C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
    "scft_field_read": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_int), _dp, _dp, _dp, _dp]),
    "scft_field_write": (C.c_int, [C.c_char_p, C.c_int, _dp, _dp, C.c_double, C.c_double]),
    "scft_res_read": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_int), _dp, C.POINTER(C.c_int),
                                C.POINTER(C.c_int), _dp]),
}

_lib = None


def load(path: str | None = None):
    """Load libscft.so (once).  Raises ImportError when it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"libscft.so not found at {p}: run __graft_entry__.build() "
                          "(python -m scft_gb300.build); there is no CPU fallback")
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class ScftError(RuntimeError):
    def __init__(self, code: int, where: str):
        lib = load()
        msg = (lib.scft_last_error().decode() or lib.scft_ws_last_error().decode()
               or lib.scft_strerror(code).decode())
        super().__init__(f"{where}: {msg} (code {code})")
        self.code = code


def check(code: int, where: str) -> int:
    if code < 0:
        raise ScftError(code, where)
    return code
