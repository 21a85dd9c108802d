"""ctypes binding of libsfhgpu.so (the C ABI in include/sfhgpu.h).

The library is the only compute path: if it is missing or cannot be loaded,
every entry point raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

_PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(_PKG_ROOT, "_build", "libsfhgpu.so")

SFH_OK, SFH_ERR_ARG, SFH_ERR_SHAPE, SFH_ERR_CUDA, SFH_ERR_TIMEOUT, SFH_ERR_NOMEM, \
    SFH_ERR_UNSUPPORTED, SFH_ERR_NUMERIC = range(8)
SFH_F64, SFH_F32, SFH_BF16X2 = 0, 1, 2
SFH_INJECT_NONE, SFH_INJECT_DROP_COPY, SFH_INJECT_ALLOC_FAIL = 0, 1, 2
SFH_HOST_ACCESS_AUTO, SFH_HOST_ACCESS_STAGED, SFH_HOST_ACCESS_DIRECT = -1, 0, 1
SFH_OCC_OFF, SFH_OCC_AUTO, SFH_OCC_ON = 0, 1, 2

# Every symbol declared in include/sfhgpu.h.
EXPORTED = [
    "sfh_abi_version", "sfh_status_string", "sfh_ctx_create", "sfh_ctx_destroy",
    "sfh_ctx_last_error", "sfh_ctx_synchronize", "sfh_ctx_stream", "sfh_ctx_launch_count",
    "sfh_ctx_set_wait_budget", "sfh_ctx_inject_fault", "sfh_ctx_set_host_access", "sfh_ctx_set_overlap",
    "sfh_ctx_host_access",
    "sfh_models_upload", "sfh_models_from_device", "sfh_models_free", "sfh_models_info",
    "sfh_models_combine",
    "sfh_composite", "sfh_loglikelihood", "sfh_grad_loglikelihood", "sfh_fg", "sfh_fg_dev",
    "sfh_fg_batched_dev", "sfh_fg_kernel_times", "sfh_models_autotune", "sfh_models_set_path", "sfh_models_set_onepass_tile",
    "sfh_models_set_onepass_ctas", "sfh_models_set_onepass_schedule", "sfh_models_onepass_variant", "sfh_models_set_onepass_run",
    "sfh_models_set_occupied", "sfh_models_occupied_info",
    "sfh_models_path", "sfh_fg_dev_noalloc", "sfh_hmc_sample_dev", "sfh_nuts_sample_dev",
    "sfh_logdensity_batched_dev", "sfh_fit_sfh_dev", "sfh_model_cmd", "sfh_model_cmd_dev", "sfh_fit_bfgs", "sfh_fit_bfgs_dev", "sfh_bin_cmd", "sfh_bin_cmd_dev", "sfh_bin_cmd_smooth", "sfh_bin_cmd_smooth_batch_dev",
    "sfh_partial_cmd_smooth_batch_dev", "sfh_partial_cmd_smooth_ragged_dev",
    "sfh_binary_hess_batch_dev", "sfh_mix_binary_templates_dev",
    "sfh_galaxies_create", "sfh_galaxies_free", "sfh_galaxies_info", "sfh_fg_ragged_dev",
    "sfh_mlp_param_count", "sfh_mlp_forward",
    "sfh_mlp_loss_grad", "sfh_mlp_train", "sfh_mlp_train_grouped", "sfh_mlp_forward_rows",
    "sfh_gemm_f32", "sfh_emu_prepare", "sfh_emu_reconstruct", "sfh_emu_reconstruct_rows",
    "sfh_emu_reconstruct_groups",
    "sfh_poisson_deviance",
]


class ErrModel(C.Structure):
    """exp_photerr(m, a, b, c, d) capped at ``cap`` (src/utilities.jl:218)."""
    _fields_ = [("a", C.c_double), ("b", C.c_double), ("c", C.c_double), ("d", C.c_double),
                ("cap", C.c_double)]


class FitOptions(C.Structure):
    """sfh_fit_options (device BFGS driver)."""
    _fields_ = [("transform", C.c_int), ("max_iter", C.c_int), ("max_evals", C.c_int),
                ("graph_slots", C.c_int), ("g_abstol", C.c_double), ("f_reltol", C.c_double),
                ("x_abstol", C.c_double), ("eps", C.c_double)]


class FitResult(C.Structure):
    """sfh_fit_result (device BFGS driver)."""
    _fields_ = [("f", C.c_double), ("g_norm", C.c_double), ("iterations", C.c_int64),
                ("evaluations", C.c_int64), ("status", C.c_int), ("graph", C.c_int)]


class ComplModel(C.Structure):
    """Martin2016_complete(m, A, m50, rho) (src/utilities.jl:205)."""
    _fields_ = [("A", C.c_double), ("m50", C.c_double), ("rho", C.c_double)]


class IMFParams(C.Structure):
    _fields_ = [("nseg", C.c_int32), ("mmin", C.c_double), ("mmax", C.c_double),
                ("breaks", C.c_double * 3), ("alpha", C.c_double * 4)]


class SFHError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(message)
        self.status = status


class SFHArgumentError(SFHError, ValueError):
    """Raised where the reference's @argcheck throws ArgumentError."""


_lib = None
_lock = threading.Lock()
_vp = C.c_void_p
_i64 = C.c_int64
_d = C.c_double


def load(path: str | None = None):
    """Load libsfhgpu.so (building it first when the toolkit is present)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            try:
                import importlib.util
                spec = importlib.util.spec_from_file_location(
                    "_sfh_build", os.path.join(_PKG_ROOT, "build.py"))
                mod = importlib.util.module_from_spec(spec)
                spec.loader.exec_module(mod)
                mod.build()
            except Exception as e:  # noqa: BLE001 - re-raised with context
                raise SFHError(SFH_ERR_UNSUPPORTED,
                               f"libsfhgpu.so is not built and building failed: {e}") from e
        L = C.CDLL(p)
        sig = {
            "sfh_abi_version": ([], C.c_int),
            "sfh_status_string": ([C.c_int], C.c_char_p),
            "sfh_ctx_create": ([C.c_int, C.POINTER(_vp)], C.c_int),
            "sfh_ctx_destroy": ([_vp], C.c_int),
            "sfh_ctx_last_error": ([_vp], C.c_char_p),
            "sfh_ctx_synchronize": ([_vp], C.c_int),
            "sfh_ctx_stream": ([_vp, C.POINTER(_vp)], C.c_int),
            "sfh_ctx_launch_count": ([_vp, C.POINTER(_i64)], C.c_int),
            "sfh_ctx_set_wait_budget": ([_vp, _i64], C.c_int),
            "sfh_ctx_inject_fault": ([_vp, C.c_int], C.c_int),
            "sfh_ctx_set_host_access": ([_vp, C.c_int], C.c_int),
            "sfh_ctx_set_overlap": ([_vp, C.c_int], C.c_int),
            "sfh_ctx_host_access": ([_vp, C.POINTER(C.c_int)], C.c_int),
            "sfh_models_upload": ([_vp, _vp, C.c_int, _i64, _i64, C.c_int, C.POINTER(_vp)], C.c_int),
            "sfh_models_from_device": ([_vp, _vp, _i64, _i64, C.c_int, C.POINTER(_vp)], C.c_int),
            "sfh_models_free": ([_vp], C.c_int),
            "sfh_models_combine": ([_vp, _vp, _i64, _vp, _vp, _vp, C.c_int, C.POINTER(_vp)],
                                   C.c_int),
            "sfh_models_info": ([_vp, C.POINTER(_i64), C.POINTER(_i64), C.POINTER(C.c_int)],
                                C.c_int),
            "sfh_composite": ([_vp, _vp, C.c_int, _vp, _vp], C.c_int),
            "sfh_loglikelihood": ([_vp, C.c_int, _vp, _vp, _i64, C.POINTER(_d)], C.c_int),
            "sfh_grad_loglikelihood": ([_vp, _vp, C.c_int, _vp, _vp, _vp], C.c_int),
            "sfh_fg": ([_vp, _vp, C.c_int, _vp, _vp, _vp, _vp, C.POINTER(_d)], C.c_int),
            "sfh_fg_dev": ([_vp, _vp, _vp, _vp, _vp, _vp, _vp, _d], C.c_int),
            "sfh_fg_batched_dev": ([_vp, _vp, _vp, _i64, _vp, _vp, _vp, _d], C.c_int),
            "sfh_models_autotune": ([_vp, _vp, _vp, _vp, _d, C.c_int, _vp, _vp], C.c_int),
            "sfh_models_set_path": ([_vp, _vp, C.c_int], C.c_int),
            "sfh_models_set_onepass_tile": ([_vp, _vp, C.c_int], C.c_int),
            "sfh_models_set_onepass_ctas": ([_vp, _vp, C.c_int], C.c_int),
            "sfh_models_set_onepass_schedule": ([_vp, _vp, C.c_int], C.c_int),
            "sfh_models_onepass_variant": ([_vp, _vp, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                            C.POINTER(C.c_int), C.POINTER(C.c_int)], C.c_int),
            "sfh_models_set_onepass_run": ([_vp, _vp, C.c_int], C.c_int),
            "sfh_models_set_occupied": ([_vp, _vp, C.c_int], C.c_int),
            "sfh_models_occupied_info": ([_vp, _vp, _vp, C.POINTER(_i64), C.POINTER(C.c_int),
                                          C.POINTER(_d)], C.c_int),
            "sfh_models_path": ([_vp, _vp, C.POINTER(C.c_int), C.POINTER(_d)], C.c_int),
            "sfh_fg_dev_noalloc": ([_vp, _vp, _i64, _i64, _vp, _vp, _vp, _vp, _vp, _d], C.c_int),
            "sfh_fg_kernel_times": ([_vp, _vp, _vp, _vp, _vp, _vp, _vp, _d, C.c_int,
                                     C.POINTER(_d)], C.c_int),
            "sfh_model_cmd": ([_vp, _vp, _vp, _vp, _vp, _i64, C.c_int, C.c_uint64, _vp, _vp,
                               C.POINTER(_i64)], C.c_int),
            "sfh_model_cmd_dev": ([_vp, _vp, _vp, _vp, _vp, _i64, C.c_int, C.c_uint64, _vp, _vp,
                                   C.POINTER(_i64)], C.c_int),
            "sfh_fit_bfgs": ([_vp, _vp, _vp, _vp, C.POINTER(FitOptions), _vp, _vp,
                              C.POINTER(FitResult)], C.c_int),
            "sfh_fit_bfgs_dev": ([_vp, _vp, _vp, _vp, C.POINTER(FitOptions), _vp, _vp,
                                  C.POINTER(FitResult)], C.c_int),
            "sfh_bin_cmd": ([_vp, _vp, _vp, _vp, _i64, _vp, _i64, _vp, _i64, _vp], C.c_int),
            "sfh_bin_cmd_dev": ([_vp, _vp, _vp, _vp, _i64, _vp, _i64, _vp, _i64, _vp], C.c_int),
            "sfh_bin_cmd_smooth": ([_vp] + [_vp] * 5 + [_i64, C.c_int, _d, _d, _i64, _d, _d, _i64,
                                                         _vp], C.c_int),
            "sfh_bin_cmd_smooth_batch_dev": ([_vp] + [_vp] * 6 + [_vp, _i64, _d, _d, _i64, _d, _d,
                                                                   _i64, _vp], C.c_int),
            "sfh_partial_cmd_smooth_batch_dev": (
                [_vp, _vp, _vp, _i64, _vp, _vp, _i64, C.c_int, C.c_int, C.c_int, C.c_int,
                 C.POINTER(ErrModel), C.POINTER(ComplModel), _vp, C.POINTER(IMFParams), _d, _vp,
                 _vp, _d, _d, _i64, _d, _d, _i64, _vp], C.c_int),
            "sfh_binary_hess_batch_dev": (
                [_vp, _vp, _vp, _i64, _vp, _vp, _i64, C.c_int, C.c_int, C.c_int, C.c_int,
                 C.POINTER(ErrModel), C.POINTER(ComplModel), _vp, C.POINTER(IMFParams), _d, _vp,
                 _d, _d, _i64, _d, _d, _i64, _vp], C.c_int),
            "sfh_mix_binary_templates_dev": ([_vp, _vp, _vp, _vp, _i64, _i64, _vp], C.c_int),
            "sfh_partial_cmd_smooth_ragged_dev": (
                [_vp, _vp, _vp, _i64, _vp, _vp, _i64, C.c_int, C.c_int, C.c_int, C.c_int,
                 C.POINTER(ErrModel), C.POINTER(ComplModel), _vp, C.POINTER(IMFParams), _d, _vp,
                 _vp, _vp, _i64, _vp], C.c_int),
            "sfh_galaxies_create": ([_vp, _vp, _i64, _vp, _i64, C.POINTER(_vp)], C.c_int),
            "sfh_galaxies_free": ([_vp], C.c_int),
            "sfh_galaxies_info": ([_vp, C.POINTER(_i64), C.POINTER(_i64), C.POINTER(_i64)],
                                  C.c_int),
            "sfh_fg_ragged_dev": ([_vp, _vp, _vp, _vp, _vp, _vp, _vp, _d], C.c_int),
            "sfh_mlp_param_count": ([C.c_int] * 4 + [C.POINTER(_i64)], C.c_int),
            "sfh_mlp_forward": ([_vp] + [C.c_int] * 4 + [_vp, _vp, C.c_int, _vp], C.c_int),
            "sfh_mlp_loss_grad": ([_vp] + [C.c_int] * 4 + [_vp, _vp, _vp, C.c_int, _vp, _vp],
                                  C.c_int),
            "sfh_mlp_train": ([_vp] + [C.c_int] * 4 + [_vp, _vp, _vp, _i64, _vp, _vp, _i64,
                                                       C.c_int, _i64, C.c_float, C.c_uint64,
                                                       _vp], C.c_int),
            "sfh_mlp_train_grouped": ([_vp] + [C.c_int] * 4 + [_i64, _vp, _vp, _vp, _i64, _vp, _vp,
                                                                _vp, C.c_int, _i64, C.c_float,
                                                                C.c_uint64, _vp], C.c_int),
            "sfh_mlp_forward_rows": ([_vp] + [C.c_int] * 4 + [_vp, _i64, _vp, _vp, _i64, _vp],
                                     C.c_int),
            "sfh_emu_reconstruct_rows": ([_vp, _vp, _vp, _i64, _vp, _vp, C.c_int, _i64, _i64,
                                          C.c_int, _vp], C.c_int),
            "sfh_emu_reconstruct_groups": ([_vp, _vp, _vp, _vp, _i64, _i64, _vp, _vp, C.c_int,
                                            _i64, _i64, C.c_int, _vp], C.c_int),
            "sfh_gemm_f32": ([_vp, _vp, _vp, _vp, _i64, _i64, _i64, C.c_int, C.c_int, C.c_int,
                              C.c_float, C.c_int], C.c_int),
            "sfh_emu_prepare": ([_vp, _vp, _i64, _i64, C.c_int, _vp], C.c_int),
            "sfh_emu_reconstruct": ([_vp, _vp, _vp, _vp, C.c_int, _i64, _i64, C.c_int, _vp],
                                    C.c_int),
            "sfh_poisson_deviance": ([_vp, _vp, _vp, _i64, C.c_int, _vp], C.c_int),
        }
        for name, (args, res) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
        return _lib


def status_string(code: int) -> str:
    return load().sfh_status_string(code).decode()


def check(rc: int, ctx_ptr=None, what: str = ""):
    if rc == SFH_OK:
        return
    L = load()
    msg = L.sfh_status_string(rc).decode()
    if ctx_ptr:
        detail = L.sfh_ctx_last_error(ctx_ptr).decode()
        if detail:
            msg = f"{msg}: {detail}"
    if what:
        msg = f"{what}: {msg}"
    if rc in (SFH_ERR_ARG, SFH_ERR_SHAPE):
        raise SFHArgumentError(rc, msg)
    raise SFHError(rc, msg)


def ptr(a) -> int | None:
    """Address of a numpy array or torch tensor (host or device), or None."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    if isinstance(a, int):
        return a
    raise TypeError(f"cannot take the address of {type(a)}")
