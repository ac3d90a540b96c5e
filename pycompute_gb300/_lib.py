"""ctypes binding of libpcgb.so (the C ABI declared in include/pcgb.h).

The library is built in-tree by ``pycompute_gb300.build``. Loading it is
mandatory: if it is missing or fails to load, every fitter call raises; there
is no Python or PyTorch fallback for the fitting kernels.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None

c_int, c_i64, c_double, c_void_p, c_char_p, c_size_t = (ctypes.c_int, ctypes.c_int64, ctypes.c_double,
                                                        ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t)

# name -> (restype, argtypes); exactly the entry points of include/pcgb.h
SIGNATURES = {
    "pcgb_version": (c_char_p, []),
    "pcgb_max_params": (c_int, []),
    "pcgb_max_protocol": (c_int, []),
    "pcgb_last_error": (c_char_p, []),
    "pcgb_fitter_create": (c_int, [c_char_p, c_char_p, c_int, c_int, c_int, c_int, c_int, c_char_p,
                                   ctypes.POINTER(c_void_p)]),
    "pcgb_fitter_compile": (c_int, [c_char_p, c_char_p, c_int, c_int, c_int, c_int, c_int, c_char_p, c_char_p,
                                    c_size_t]),
    "pcgb_fitter_destroy": (c_int, [c_void_p]),
    "pcgb_fitter_log": (c_char_p, [c_void_p]),
    "pcgb_lm_run": (c_int, [c_void_p, c_void_p, c_i64, c_void_p, c_void_p, c_void_p, c_i64, c_double, c_double,
                            c_double, c_double, c_double, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                            c_void_p, c_void_p, c_i64, c_int, c_void_p, c_int, c_void_p, c_void_p, c_int,
                            c_void_p]),
    "pcgb_lm_run_subset": (c_int, [c_void_p, c_void_p, c_i64, c_void_p, c_void_p, c_void_p, c_i64, c_double,
                                   c_double, c_double, c_double, c_double, c_void_p, c_void_p, c_void_p, c_void_p,
                                   c_void_p, c_void_p, c_void_p, c_void_p, c_i64, c_int, c_void_p, c_int, c_void_p,
                                   c_void_p, c_int, c_void_p, c_i64, c_void_p, c_void_p]),
    "pcgb_lm_run_fresh": (c_int, [c_void_p, c_void_p, c_i64, c_void_p, c_void_p, c_void_p, c_i64, c_double, c_double,
                                  c_double, c_double, c_double, c_void_p, c_void_p, c_i64, c_int, c_void_p, c_int,
                                  c_void_p, c_void_p, c_double, c_int, c_void_p]),
    "pcgb_lm_run_refill": (c_int, [c_void_p, c_void_p, c_i64, c_void_p, c_void_p, c_void_p, c_i64, c_double,
                                   c_double, c_double, c_double, c_double, c_void_p, c_void_p, c_void_p, c_void_p,
                                   c_void_p, c_void_p, c_void_p, c_void_p, c_i64, c_int, c_void_p, c_int, c_void_p,
                                   c_void_p, c_int, c_void_p, c_i64, c_void_p, c_void_p, c_int, c_void_p]),
    "pcgb_lm_run_check": (c_int, [c_void_p, c_void_p, c_i64, c_void_p, c_void_p, c_void_p, c_i64, c_double,
                                  c_double, c_double, c_double, c_double, c_void_p, c_void_p, c_void_p, c_void_p,
                                  c_void_p, c_void_p, c_void_p, c_void_p, c_i64, c_int, c_void_p, c_int, c_void_p,
                                  c_void_p, c_int, c_void_p, c_double, c_void_p, c_void_p, c_void_p, c_void_p,
                                  c_void_p, c_void_p]),
    "pcgb_lm_run_select": (c_int, [c_void_p, c_void_p, c_i64, c_void_p, c_void_p, c_void_p, c_i64, c_double,
                                   c_double, c_double, c_double, c_double, c_void_p, c_void_p, c_void_p, c_void_p,
                                   c_void_p, c_void_p, c_void_p, c_void_p, c_i64, c_int, c_void_p, c_int, c_void_p,
                                   c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                   c_void_p]),
    "pcgb_warm_check": (c_int, [c_void_p, c_void_p, c_i64, c_void_p, c_void_p, c_void_p, c_i64, c_void_p, c_int,
                                c_void_p, c_void_p, c_void_p, c_double, c_void_p, c_void_p, c_void_p, c_void_p,
                                c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_i64, c_void_p]),
    "pcgb_warm_lm_check": (c_int, [c_void_p, c_void_p, c_i64, c_void_p, c_void_p, c_void_p, c_i64, c_double,
                                   c_double, c_double, c_double, c_double, c_int, c_double, c_void_p, c_int, c_void_p,
                                   c_void_p, c_void_p, c_double, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                   c_void_p, c_void_p, c_void_p, c_void_p, c_i64, c_int, c_void_p]),
    "pcgb_warm_select": (c_int, [c_void_p, c_void_p, c_i64, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p,
                                 c_void_p, c_void_p, c_void_p, c_void_p, c_i64, c_void_p]),
    "pcgb_f_run_subset": (c_int, [c_void_p, c_void_p, c_void_p, c_i64, c_void_p, c_void_p, c_void_p, c_i64,
                                  c_void_p, c_int, c_void_p, c_i64, c_void_p]),
    "pcgb_f_run": (c_int, [c_void_p, c_void_p, c_void_p, c_i64, c_void_p, c_void_p, c_void_p, c_i64, c_void_p,
                           c_int, c_void_p]),
    "pcgb_gmw81_solve": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_i64, c_void_p]),
    "pcgb_search_step": (c_int, [c_void_p, c_void_p, c_i64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_i64,
                                 c_void_p, c_int, c_void_p]),
    "pcgb_random_search": (c_int, [c_void_p, c_void_p, c_i64, c_void_p, c_void_p, c_void_p, c_i64, c_void_p,
                                   c_void_p, c_i64, c_int, c_int, c_double, c_double, c_double, c_double, c_double,
                                   ctypes.c_uint64, c_void_p, c_int, c_void_p, c_void_p, c_void_p]),
    "pcgb_multi_create": (c_int, [c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_int,
                                  c_void_p, c_char_p, ctypes.POINTER(c_void_p)]),
    "pcgb_multi_destroy": (c_int, [c_void_p]),
    "pcgb_multi_log": (c_char_p, [c_void_p]),
    "pcgb_multi_grid": (c_int, [c_void_p]),
    "pcgb_multi_run": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_int, c_double, c_double, c_double, c_double,
                               c_double, c_int, c_int, c_void_p, c_void_p]),
    "pcgb_multi_run_noalloc": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_int, c_double, c_double, c_double,
                                       c_double, c_double, c_int, c_int, c_void_p]),
    "pcgb_noalloc_last_error": (c_char_p, []),
    "pcgb_model_eval": (c_int, [c_void_p, c_void_p, c_void_p, c_i64, c_void_p, c_i64, c_void_p, c_int, c_void_p]),
    "pcgb_pipeline_last_error": (c_char_p, []),
    "pcgb_fp64_helpers": (c_int, [c_void_p, c_void_p, c_void_p, c_i64, c_void_p]),
    "pcgb_copy_rows_async": (c_int, [c_void_p, c_i64, c_void_p, c_i64, c_i64, c_i64, c_int, c_void_p]),
    "pcgb_init_constant": (c_int, [c_void_p, c_i64, c_int, c_int, c_void_p, c_void_p, c_void_p]),
    "pcgb_bpolyfit": (c_int, [c_void_p, c_i64, c_void_p, c_void_p, c_i64, c_int, c_int, c_int, c_int, c_void_p,
                              c_void_p]),
    "pcgb_ivim_segmented_init": (c_int, [c_void_p, c_void_p, c_i64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                         c_void_p]),
    "pcgb_fallback_flags": (c_int, [c_void_p, c_void_p, c_void_p, c_i64, c_int, c_void_p, c_void_p, c_void_p,
                                    c_void_p, c_void_p, c_void_p]),
    "pcgb_fallback_prepare": (c_int, [c_void_p, c_i64, c_i64, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                      c_void_p, c_void_p, c_void_p, ctypes.c_float, c_void_p, c_void_p, c_void_p]),
    "pcgb_fallback_select": (c_int, [c_void_p, c_i64, c_i64, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                     c_void_p, c_void_p]),
    "pcgb_mlp_last_error": (c_char_p, []),
    "pcgb_gemm_bf16": (c_int, [c_int, c_int, c_int, c_void_p, c_i64, c_void_p, c_i64, c_i64, c_i64, c_i64, c_i64,
                               c_void_p, c_i64, c_void_p, c_i64, c_void_p, c_i64, c_void_p, c_i64, c_void_p]),
    "pcgb_gemm_bf16_tc": (c_int, [c_int, c_int, c_int, c_void_p, c_i64, c_void_p, c_i64, c_i64, c_i64, c_i64,
                                  c_i64, c_void_p, c_i64, c_void_p, c_i64, c_void_p, c_i64, c_void_p, c_i64, c_void_p,
                                  c_void_p]),
    "pcgb_gemm_bf16_tc_ex": (c_int, [c_int, c_int, c_int, c_void_p, c_i64, c_void_p, c_i64, c_i64, c_i64, c_i64,
                                     c_i64, c_void_p, c_i64, c_void_p, c_i64, c_void_p, c_i64, c_void_p, c_i64,
                                     c_void_p, ctypes.c_uint, c_i64, c_void_p]),
    "pcgb_gemm_tc_last_error": (c_char_p, []),
    "pcgb_mlp_mse_grad": (c_int, [c_void_p, c_void_p, c_i64, c_i64, c_int, c_int, c_void_p, c_i64, c_void_p,
                                  c_void_p]),
    "pcgb_adam_step": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_i64, c_i64, c_i64, ctypes.c_float,
                               ctypes.c_float, ctypes.c_float, ctypes.c_float, c_void_p, c_void_p]),
    "pcgb_mlp_prepare": (c_int, [c_void_p, c_i64, c_int, c_int, c_void_p, c_i64, c_void_p, c_void_p, c_int, c_void_p,
                                 c_void_p, c_void_p, c_void_p, c_i64, c_void_p]),
    "pcgb_mlp_gelu": (c_int, [c_void_p, c_i64, c_int, c_void_p, c_void_p, c_void_p]),
    "pcgb_mlp_forward": (c_int, [c_void_p, c_i64, c_int, c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p,
                                 c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "pcgb_mlp_forward_tc": (c_int, [c_void_p, c_i64, c_int, c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p,
                                    c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "pcgb_mlp_forward_tc_ex": (c_int, [c_void_p, c_i64, c_int, c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p,
                                       c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, ctypes.c_uint, c_i64,
                                       c_void_p]),
    "pcgb_mlp_tc_last_error": (c_char_p, []),
}


class PcgbError(RuntimeError):
    """A C-ABI call returned an error code."""

    def __init__(self, fn: str, code: int, msg: str):
        super().__init__(f"{fn} failed ({code}): {msg}")
        self.code = code


def lib(build_if_missing: bool = True):
    """The loaded library (built first if needed)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if build_if_missing:
            path = _build.build()
        if not os.path.exists(path):
            raise RuntimeError(f"native library {path} is missing: run pycompute_gb300.build.build()")
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
        return L


def check(fn_name: str, rc: int):
    if rc != 0:
        L = lib()
        if fn_name.startswith("pcgb_gemm_bf16_tc"):
            err = L.pcgb_gemm_tc_last_error
        elif fn_name.startswith("pcgb_mlp_forward_tc"):  # also pcgb_mlp_forward_tc_ex
            err = L.pcgb_mlp_tc_last_error
        elif fn_name.startswith(("pcgb_gemm", "pcgb_mlp", "pcgb_adam")):
            err = L.pcgb_mlp_last_error
        elif fn_name.startswith("pcgb_multi_run_noalloc"):
            err = L.pcgb_noalloc_last_error
        elif fn_name.startswith(("pcgb_init_constant", "pcgb_fp64_helpers", "pcgb_copy_rows", "pcgb_fallback", "pcgb_bpolyfit", "pcgb_ivim")):
            err = L.pcgb_pipeline_last_error
        else:
            err = L.pcgb_last_error
        msg = err().decode(errors="replace")
        raise PcgbError(fn_name, rc, msg)


def cache_dir() -> str:
    d = os.environ.get("PCGB_CACHE_DIR") or os.path.join(_build.BUILD, "jit")
    os.makedirs(d, exist_ok=True)
    return d
