"""ctypes binding of libhjmcva.so (the C ABI in include/hjm_cva.h).

The library is built in-tree by ``cva_hjm_cuda_gb300.build``.  There is no
fallback: if the shared library is missing or cannot be loaded, every entry
point raises.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libhjmcva.so"

HJM_OK = 0
STATUS_NAMES = {
    0: "HJM_OK",
    1: "HJM_ERR_INVALID_ARGUMENT",
    2: "HJM_ERR_UNSUPPORTED",
    3: "HJM_ERR_CUDA",
    4: "HJM_ERR_OUT_OF_MEMORY",
    5: "HJM_ERR_NOT_CONFIGURED",
    6: "HJM_ERR_NO_DEVICE",
}
PRECISION = {"fp64": 0, "mixed": 1}
MAX_TENOR = 64
N_VOL_COEF = 9

# every symbol include/hjm_cva.h and include/hjm_dropin.h declare (C linkage)
EXPORTED = [
    "hjm_version", "hjm_last_error", "hjm_ctx_create", "hjm_ctx_destroy", "hjm_ctx_set_stream",
    "hjm_ctx_keep_exposures", "hjm_ctx_set_memory_limit", "hjm_ctx_memory_in_use", "hjm_ctx_set_vol_decomposition", "hjm_ctx_set_scheme", "hjm_ctx_vol_decomposition",
    "hjm_ctx_set_remainder_form", "hjm_ctx_remainder_form", "hjm_set_market", "hjm_set_swap", "hjm_set_netting_set", "hjm_run",
    "hjm_enqueue", "hjm_fetch_results", "hjm_run_with_normals", "hjm_get_exposures", "hjm_get_exposure_paths", "hjm_set_market_poly", "hjm_calibrate_pca", "hjm_write_report", "hjm_run_mlmc",
    "hjm_run_adjoint", "hjm_dump_normals", "hjm_philox_words", "hjm_last_timings", "hjm_timing_history", "hjm_last_stats", "hjm_measure_fma_peak",
    "hjm_dropin_calculate_exposure_fp64", "hjm_dropin_calculate_exposure_fp32", "hjm_run_static",
]
STATIC_MAX_PATHS = 1048576
RESPONSE_MAX_DATES = 24

_lock = threading.Lock()
_lib: C.CDLL | None = None

_dp = C.POINTER(C.c_double)
_vp = C.c_void_p


def _declare(lib: C.CDLL) -> None:
    st = C.c_int
    sigs = {
        "hjm_version": (C.c_char_p, []),
        "hjm_last_error": (C.c_char_p, [_vp]),
        "hjm_ctx_create": (st, [C.c_int, C.POINTER(_vp)]),
        "hjm_ctx_destroy": (st, [_vp]),
        "hjm_ctx_set_stream": (st, [_vp, _vp]),
        "hjm_ctx_keep_exposures": (st, [_vp, C.c_int32]),
        "hjm_ctx_set_memory_limit": (st, [_vp, C.c_int64]),
        "hjm_ctx_memory_in_use": (st, [_vp, C.POINTER(C.c_int64)]),
        "hjm_ctx_set_vol_decomposition": (st, [_vp, C.c_int32]),
        "hjm_ctx_set_scheme": (st, [_vp, C.c_int32]),
        "hjm_ctx_set_remainder_form": (st, [_vp, C.c_int32]),
        "hjm_ctx_remainder_form": (st, [_vp, C.POINTER(C.c_int32)]),
        "hjm_ctx_vol_decomposition": (st, [_vp, C.POINTER(C.c_int32)]),
        "hjm_set_market": (st, [_vp, C.c_int32, C.c_double, _dp, _dp, C.c_int32, _dp]),
        "hjm_set_market_poly": (st, [_vp, C.c_int32, C.c_double, _dp, _dp]),
        "hjm_write_report": (st, [_vp, C.c_char_p, C.c_int32]),
        "hjm_run_mlmc": (st, [_vp, C.c_int32, C.POINTER(C.c_int64), C.c_int32, C.c_double, C.c_uint64, C.c_double,
                              C.c_double, _dp, _dp, _dp]),
        "hjm_calibrate_pca": (st, [_dp, C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_int32, _dp, _dp, _dp,
                                   _dp]),
        "hjm_set_swap": (st, [_vp, C.c_double, C.c_double, _dp, C.c_int32]),
        "hjm_set_netting_set": (st, [_vp, C.c_int32, _dp, _dp, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
        "hjm_run": (st, [_vp, C.c_int64, C.c_int32, C.c_double, C.c_uint64, C.c_uint64, C.c_int32, C.c_double,
                         C.c_double, C.c_double, _dp, _dp, _dp]),
        "hjm_enqueue": (st, [_vp, C.c_int64, C.c_int32, C.c_double, C.c_uint64, C.c_uint64, C.c_int32, C.c_double,
                             C.c_double, C.c_double]),
        "hjm_fetch_results": (st, [_vp, _dp, _dp, _dp]),
        "hjm_run_with_normals": (st, [_vp, C.c_int64, C.c_int32, C.c_double, _dp, C.c_int32, C.c_double, C.c_double,
                                      C.c_double, _dp, _dp, _dp]),
        "hjm_get_exposures": (st, [_vp, _dp, C.c_int64]),
        "hjm_get_exposure_paths": (st, [_vp, C.c_int64, C.c_int64, _dp]),
        "hjm_run_adjoint": (st, [_vp, C.c_int64, C.c_int32, C.c_double, C.c_uint64, C.c_uint64, C.c_double,
                                 C.c_double, C.c_int32, _dp, _dp, _dp, _dp]),
        "hjm_dump_normals": (st, [_vp, C.c_int64, C.c_uint64, C.c_int32, C.c_uint64, _dp]),
        "hjm_philox_words": (st, [_vp, C.c_int64, C.c_uint64, C.c_uint32, C.c_uint64, C.POINTER(C.c_uint32)]),
        "hjm_last_timings": (st, [_vp, _dp]),
        "hjm_timing_history": (st, [_vp, C.c_int32, _dp]),
        "hjm_last_stats": (st, [_vp, C.POINTER(C.c_int64)]),
        "hjm_measure_fma_peak": (st, [_vp, C.c_int32, _dp]),
        "hjm_run_static": (st, [_vp, C.c_int32, C.c_double, _dp, _dp, _dp, C.c_double, C.c_double, _dp, C.c_int32,
                                C.c_int64, C.c_int32, C.c_double, C.c_uint64, C.c_uint64, C.c_int32, C.c_double,
                                C.c_double, _dp, _dp]),
        "hjm_dropin_calculate_exposure_fp64": (None, [_dp, C.c_double, C.c_double, C.c_double, C.c_double, _dp, _dp,
                                                      _dp, _dp, C.c_int, C.c_int, C.c_double]),
        "hjm_dropin_calculate_exposure_fp32": (None, [C.POINTER(C.c_float), C.c_float, C.c_float, C.c_float,
                                                      C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                                      C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int, C.c_int,
                                                      C.c_float]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


def load() -> C.CDLL:
    """Load libhjmcva.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(
                    f"{LIB_PATH} is missing: build it with `python -m cva_hjm_cuda_gb300.build` "
                    "(the engine has no CPU fallback)"
                )
            lib = C.CDLL(str(LIB_PATH))
            _declare(lib)
            _lib = lib
        return _lib


class HJMError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def check(status: int, ctx=None) -> None:
    if status != HJM_OK:
        msg = load().hjm_last_error(ctx)
        raise HJMError(status, msg.decode() if msg else "")
