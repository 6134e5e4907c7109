"""ctypes bindings of the engine's C ABI (include/hexo_mc.h).

The library is the only compute path: importing works without it, but every
call raises ``EngineUnavailable`` when libhexo_mc.so has not been built.
With HEXO_LIB=checks in the environment the bindings load the bounds-checked
build of the same sources, libhexo_mc_checks.so, instead.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

VARIANTS = {"": "libhexo_mc.so", "checks": "libhexo_mc_checks.so"}
LIB_PATH = Path(__file__).resolve().parent / VARIANTS.get(os.environ.get("HEXO_LIB", ""), "libhexo_mc.so")

HEXO_OK = 0
HEXO_ERR_TIMEOUT = 5
HEXO_ERR_NOT_FOUND = 7
HEXO_ERR_ADMISSION = 8
HEXO_ERR_SHUTDOWN = 9
HEXO_ERR_CHECK = 11
HEXO_LIMBS = 6
STATUS_NAMES = {
    0: "HEXO_OK", 1: "HEXO_ERR_INVALID", 2: "HEXO_ERR_CUDA", 3: "HEXO_ERR_NOMEM",
    4: "HEXO_ERR_UNSUPPORTED", 5: "HEXO_ERR_TIMEOUT", 6: "HEXO_ERR_NUMERIC",
    7: "HEXO_ERR_NOT_FOUND", 8: "HEXO_ERR_ADMISSION", 9: "HEXO_ERR_SHUTDOWN", 10: "HEXO_ERR_TOO_LARGE",
    11: "HEXO_ERR_CHECK",
}


class EngineUnavailable(RuntimeError):
    pass


class HexoError(RuntimeError):
    def __init__(self, status: int, message: str = ""):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


class hexo_params(C.Structure):
    _fields_ = [("v0", C.c_double), ("theta", C.c_double), ("rho", C.c_double), ("kappa", C.c_double),
                ("sigma", C.c_double), ("r", C.c_double), ("q", C.c_double)]


class hexo_option(C.Structure):
    _fields_ = [("strike", C.c_double), ("T", C.c_double), ("payoff", C.c_uint32), ("reserved", C.c_uint32),
                ("n_paths", C.c_uint64)]


class hexo_mc_cfg(C.Structure):
    _fields_ = [("n_paths", C.c_uint64), ("step_mode", C.c_uint32), ("steps", C.c_uint32),
                ("steps_per_year", C.c_double), ("seed", C.c_uint32), ("rng_block_words", C.c_uint32),
                ("precision", C.c_uint32), ("block", C.c_uint32), ("paths_per_thread", C.c_uint32),
                ("unroll", C.c_uint32), ("control_variate", C.c_uint32), ("stream", C.c_uint32)]


class hexo_ctx_opts(C.Structure):
    _fields_ = [("device", C.c_int), ("mem_cap_bytes", C.c_uint64), ("autotune_cache", C.c_char_p),
                ("flags", C.c_uint32)]


class hexo_request(C.Structure):
    _fields_ = [("params", hexo_params), ("S0", C.c_double), ("opts", C.POINTER(hexo_option)),
                ("n_opts", C.c_uint32), ("seed", C.c_uint32), ("price_out", C.POINTER(C.c_double)),
                ("stderr_out", C.POINTER(C.c_double)), ("stream", C.c_uint32), ("reserved", C.c_uint32)]


class hexo_batch_info(C.Structure):
    _fields_ = [("nominal_path_steps", C.c_uint64), ("executed_path_steps", C.c_uint64), ("n_paths", C.c_uint64),
                ("n_tiles", C.c_uint32), ("n_sets", C.c_uint32), ("n_options", C.c_uint32), ("block", C.c_uint32),
                ("paths_per_thread", C.c_uint32), ("unroll", C.c_uint32), ("grid", C.c_uint32),
                ("device_bytes", C.c_uint64), ("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64),
                ("last_kernel_ms", C.c_double), ("quad_steps", C.c_uint64)]


class hexo_plan_stats(C.Structure):
    _fields_ = [("nominal_path_steps", C.c_uint64), ("executed_path_steps", C.c_uint64), ("n_paths", C.c_uint64),
                ("n_maturities", C.c_uint32), ("n_segments", C.c_uint32), ("n_tiles", C.c_uint32),
                ("n_options", C.c_uint32)]


class hexo_tune_result(C.Structure):
    _fields_ = [("block", C.c_uint32), ("paths_per_thread", C.c_uint32), ("unroll", C.c_uint32),
                ("n_tried", C.c_uint32), ("best_ms", C.c_double)]


class hexo_tune_entry(C.Structure):
    _fields_ = [("block", C.c_uint32), ("paths_per_thread", C.c_uint32), ("unroll", C.c_uint32),
                ("ms", C.c_float)]


class hexo_server_opts(C.Structure):
    _fields_ = [("cfg", hexo_mc_cfg), ("mem_cap_bytes", C.c_uint64), ("max_batch_requests", C.c_uint32),
                ("max_inflight", C.c_uint32), ("launch_path_steps", C.c_uint64)]


class hexo_server_stats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("admitted", C.c_uint64), ("completed", C.c_uint64),
                ("failed", C.c_uint64), ("batches", C.c_uint64), ("chunks", C.c_uint64), ("queued_now", C.c_uint64),
                ("queued_max", C.c_uint64), ("inflight_now", C.c_uint64), ("mem_in_use", C.c_uint64),
                ("mem_peak", C.c_uint64), ("nominal_path_steps", C.c_uint64), ("busy_seconds", C.c_double),
                ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("mean_ms", C.c_double)]


class hexo_swift_params(C.Structure):
    _fields_ = [("m", C.c_uint32), ("exp2_m", C.c_uint32), ("sqrt_exp2_m", C.c_double), ("lower", C.c_double),
                ("upper", C.c_double), ("k1", C.c_int32), ("k2", C.c_int32), ("J", C.c_uint32),
                ("reserved", C.c_uint32)]


class hexo_swift_chain(C.Structure):
    _fields_ = [("tau", C.c_double), ("strikes", C.POINTER(C.c_double)), ("n", C.c_uint32),
                ("method", C.c_uint32), ("params", C.POINTER(hexo_swift_params)),
                ("trunc_precision", C.c_double), ("price_out", C.POINTER(C.c_double)),
                ("grad_out", C.POINTER(C.c_double))]


class hexo_swift_request(C.Structure):
    _fields_ = [("params", hexo_params), ("S", C.c_double), ("chains", C.POINTER(hexo_swift_chain)),
                ("n_chains", C.c_uint32), ("reserved", C.c_uint32)]


_P = C.c_void_p
_D = C.POINTER(C.c_double)
_U64 = C.POINTER(C.c_uint64)

# name -> (restype, argtypes); every function of include/hexo_mc.h
PROTOTYPES = {
    "hexo_status_string": (C.c_char_p, [C.c_int]),
    "hexo_abi_version": (C.c_uint32, []),
    "hexo_ctx_create": (C.c_int, [C.POINTER(_P), C.POINTER(hexo_ctx_opts)]),
    "hexo_ctx_destroy": (C.c_int, [_P]),
    "hexo_ctx_trim": (C.c_int, [_P]),
    "hexo_ctx_last_error": (C.c_int, [_P, C.c_char_p, C.c_size_t]),
    "hexo_ctx_stream": (_P, [_P]),
    "hexo_mc_cfg_default": (None, [C.POINTER(hexo_mc_cfg)]),
    "hexo_price": (C.c_int, [_P, C.POINTER(hexo_params), C.c_double, C.POINTER(hexo_option), C.c_uint32,
                             C.POINTER(hexo_mc_cfg), _D, _D]),
    "hexo_price_batch": (C.c_int, [_P, C.POINTER(hexo_request), C.c_uint32, C.POINTER(hexo_mc_cfg)]),
    "hexo_batch_prepare": (C.c_int, [_P, C.POINTER(hexo_request), C.c_uint32, C.POINTER(hexo_mc_cfg),
                                     C.POINTER(_P)]),
    "hexo_batch_launch": (C.c_int, [_P]),
    "hexo_batch_collect": (C.c_int, [_P]),
    "hexo_batch_info_get": (C.c_int, [_P, C.POINTER(hexo_batch_info)]),
    "hexo_batch_destroy": (C.c_int, [_P]),
    "hexo_server_create": (C.c_int, [_P, C.POINTER(hexo_server_opts), C.POINTER(_P)]),
    "hexo_server_submit": (C.c_int, [_P, C.POINTER(hexo_request), _U64]),
    "hexo_server_poll": (C.c_int, [_P, C.c_uint64, C.POINTER(C.c_int)]),
    "hexo_server_wait": (C.c_int, [_P, C.c_uint64, C.c_uint32]),
    "hexo_server_stats_get": (C.c_int, [_P, C.POINTER(hexo_server_stats)]),
    "hexo_server_destroy": (C.c_int, [_P]),
    "hexo_swift_params_dynamic": (C.c_int, [C.POINTER(hexo_params), C.c_double, C.c_double, C.c_double, C.c_double,
                                            C.c_double, C.POINTER(hexo_swift_params)]),
    "hexo_swift_price": (C.c_int, [_P, C.POINTER(hexo_swift_request), C.c_uint32]),
    "hexo_calib_create": (C.c_int, [_P, C.c_double, C.c_double, _D, C.POINTER(C.c_uint32), _D, C.c_uint32, C.c_double,
                                    C.POINTER(_P)]),
    "hexo_calib_observations": (C.c_uint32, [_P]),
    "hexo_calib_prices": (C.c_int, [_P, _D, _D]),
    "hexo_calib_jacobian": (C.c_int, [_P, _D, _D]),
    "hexo_calib_destroy": (C.c_int, [_P]),
    "hexo_price_partial": (C.c_int, [_P, C.POINTER(hexo_params), C.c_double, C.POINTER(hexo_option), C.c_uint32,
                                     C.POINTER(hexo_mc_cfg), C.c_uint64, C.c_uint64, _U64]),
    "hexo_price_batch_partial": (C.c_int, [_P, C.POINTER(hexo_request), C.c_uint32, C.POINTER(hexo_mc_cfg),
                                           C.c_uint32, C.c_uint32, _U64]),
    "hexo_batch_prepare_partial": (C.c_int, [_P, C.POINTER(hexo_request), C.c_uint32, C.POINTER(hexo_mc_cfg),
                                             C.c_uint32, C.c_uint32, C.POINTER(_P)]),
    "hexo_batch_collect_limbs": (C.c_int, [_P, _U64]),
    "hexo_finalize_limbs": (C.c_int, [C.POINTER(hexo_params), C.c_double, C.POINTER(hexo_option), C.c_uint32,
                                      C.POINTER(hexo_mc_cfg), _U64, _D, _D]),
    "hexo_price_noalloc": (C.c_int, [C.POINTER(hexo_params), C.c_double, C.POINTER(hexo_option), C.c_uint32,
                                     C.POINTER(hexo_mc_cfg), _D, _D, _P]),
    "hexo_plan_stats_get": (C.c_int, [C.POINTER(hexo_request), C.c_uint32, C.POINTER(hexo_mc_cfg),
                                      C.POINTER(hexo_plan_stats)]),
    "hexo_plan_schedule": (C.c_int, [C.POINTER(hexo_params), C.c_double, C.POINTER(hexo_option), C.c_uint32,
                                     C.POINTER(hexo_mc_cfg), C.c_uint32, _U64, _D, _D, C.POINTER(C.c_uint32)]),
    "hexo_autotune": (C.c_int, [_P, C.POINTER(hexo_request), C.c_uint32, C.POINTER(hexo_mc_cfg),
                                C.POINTER(hexo_tune_result), C.POINTER(hexo_tune_entry), C.c_uint32]),
    "hexo_debug_rng_words": (C.c_int, [_P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, _U64]),
    "hexo_debug_rng_draws": (C.c_int, [_P, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(C.c_uint8), C.c_uint32,
                                       _D]),
    "hexo_debug_normals": (C.c_int, [_P, _U64, C.c_uint64, _D]),
    "hexo_debug_as241_check": (C.c_int, [_P, C.c_uint32, C.c_uint64, C.c_uint64, _U64]),
    "hexo_debug_payoff_limbs": (C.c_int, [_P, _D, C.c_uint64, C.c_uint32, C.c_double, C.POINTER(C.c_uint32)]),
    "hexo_debug_pipe_peaks": (C.c_int, [_P, _D]),
    "hexo_debug_path_finals": (C.c_int, [_P, C.POINTER(hexo_params), C.c_double, C.POINTER(hexo_option),
                                         C.c_uint32, C.POINTER(hexo_mc_cfg), C.c_uint64, C.c_uint64, _D, _D,
                                         C.POINTER(C.c_uint32)]),
}

_lib = None


ABI_VERSION = 4   # HEXO_ABI_VERSION of include/hexo_mc.h these prototypes and structs follow


def load() -> C.CDLL:
    """Loads libhexo_mc.so (built in-tree) and binds every prototype."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise EngineUnavailable(
            f"{LIB_PATH} is missing: build it with `python -m hestonexotics_gb300.build` "
            "(the engine has no CPU fallback)")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.hexo_abi_version() != ABI_VERSION:
        raise EngineUnavailable(f"{LIB_PATH} has ABI version {lib.hexo_abi_version()}, these bindings "
                                f"expect {ABI_VERSION}: rebuild it")
    _lib = lib
    return lib


def exported_symbols():
    return sorted(PROTOTYPES)
