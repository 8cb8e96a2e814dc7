"""ctypes binding of libnfftgb300.so (include/nfft_gb300.h).

The library is loaded from this package directory; it is built in-tree by
``nfft.jl_gb300/build.py`` (or ``__graft_entry__.build()``).  There is no
fallback: a missing library raises ``ImportError``.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libnfftgb300.so")

NFFT_OK = 0
NFFT_ERR_INVALID_ARG = 1
NFFT_ERR_DIM_MISMATCH = 2
NFFT_ERR_NODE_OUT_OF_RANGE = 3
NFFT_ERR_ALLOC = 4
NFFT_ERR_CUDA = 5
NFFT_ERR_CUFFT = 6
NFFT_ERR_TIMEOUT = 7
NFFT_ERR_UNSUPPORTED = 8
NFFT_ERR_NO_NODES = 9


class nfft_params(ctypes.Structure):
    _fields_ = [
        ("m", ctypes.c_int32),
        ("sigma", ctypes.c_double),
        ("window", ctypes.c_int32),
        ("precompute", ctypes.c_int32),
        ("blocking", ctypes.c_int32),
        ("sort_nodes", ctypes.c_int32),
        ("store_deconv_idx", ctypes.c_int32),
        ("block_size", ctypes.c_int64 * 3),
        ("compensated", ctypes.c_int32),
        ("timing", ctypes.c_int32),
    ]


class nfft_info(ctypes.Structure):
    _fields_ = [
        ("precision", ctypes.c_int32),
        ("D", ctypes.c_int32),
        ("N", ctypes.c_int64 * 3),
        ("Ntilde", ctypes.c_int64 * 3),
        ("M", ctypes.c_int64),
        ("m", ctypes.c_int32),
        ("sigma", ctypes.c_double),
        ("window", ctypes.c_int32),
        ("precompute", ctypes.c_int32),
        ("lut_size", ctypes.c_int64),
        ("block_size", ctypes.c_int64 * 3),
        ("num_tiles", ctypes.c_int64),
        ("num_spread_tasks", ctypes.c_int64),
        ("num_spread_entries", ctypes.c_int64),
        ("scratch_bytes", ctypes.c_int64),
    ]


# Every symbol the header declares, with (restype, argtypes).
_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_I64P = ctypes.POINTER(ctypes.c_int64)
_I32P = ctypes.POINTER(ctypes.c_int32)
SIGNATURES = {
    "nfft_params_default": (None, [ctypes.POINTER(nfft_params)]),
    "nfft_plan_create": (_I, [ctypes.POINTER(_P), _I, _I, _I64P, _I64, ctypes.POINTER(nfft_params), _P]),
    "nfft_plan_destroy": (_I, [_P]),
    "nfft_plan_copy": (_I, [_P, ctypes.POINTER(_P)]),
    "nfft_set_stream": (_I, [_P, _P]),
    "nfft_set_nodes": (_I, [_P, _P, _I]),
    "nfft_sort_nodes": (_I, [_I, _I, _I64, _P, _I, _P]),
    "nfft_forward": (_I, [_P, _P, _P]),
    "nfft_adjoint": (_I, [_P, _P, _P]),
    "nfft_convolve": (_I, [_P, _P, _I, _P, _I]),
    "nfft_convolve_transpose": (_I, [_P, _P, _I, _P, _I]),
    "nfft_deconvolve": (_I, [_P, _P, _P]),
    "nfft_deconvolve_transpose": (_I, [_P, _P, _P]),
    "nfft_grad_nodes": (_I, [_P, _P, _P, _P]),
    "nfft_autotune": (_I, [_P, _I]),
    "nfft_set_block_size": (_I, [_P, _I64P]),
    "nfft_get_info": (_I, [_P, ctypes.POINTER(nfft_info)]),
    "nfft_grid": (_P, [_P]),
    "nfft_get_timing": (_I, [_P, ctypes.POINTER(ctypes.c_double)]),
    "nfft_get_timing_totals": (_I, [_P, ctypes.POINTER(ctypes.c_double), _I64P]),
    "nfft_timing_reset": (_I, [_P]),
    "nfft_get_binning": (_I, [_P, _I32P, _I32P, _I32P]),
    "nfft_get_deconv_factors": (_I, [_P, _P]),
    "nfft_sync": (_I, [_P]),
    "nfft_bin_nodes_noalloc": (_I, [_I, _I, _I64P, _I64P, _I64, _P, _P, _P, _P]),
    "nfft_set_tiling": (_I, [_P, _I64P, _I]),
    "nfft_batch_create": (_I, [_P, _P, _I, _P]),
    "nfft_batch_destroy": (_I, [_P]),
    "nfft_batch_forward": (_I, [_P, _P, _P]),
    "nfft_batch_adjoint": (_I, [_P, _P, _P]),
    "nfft_dplan_create": (_I, [_P, _I, _I, _I64P, _I, _I, _I64, _P, _P]),
    "nfft_dplan_destroy": (_I, [_P]),
    "nfft_dplan_set_nodes": (_I, [_P, _P, _I]),
    "nfft_dplan_set_stream": (_I, [_P, _P]),
    "nfft_dplan_forward": (_I, [_P, _P, _P]),
    "nfft_dplan_adjoint": (_I, [_P, _P, _P]),
    "nfft_toeplitz_create": (_I, [ctypes.POINTER(_P), _I, _I, _I64P, _I, _P]),
    "nfft_toeplitz_destroy": (_I, [_P]),
    "nfft_toeplitz_set_stream": (_I, [_P, _P]),
    "nfft_toeplitz_is_fused": (_I, [_P, ctypes.POINTER(ctypes.c_int)]),
    "nfft_toeplitz_kernel": (_I, [_P, _P, _P]),
    "nfft_toeplitz_kernel_explicit": (_I, [_P, _P, _I64, _I, _P]),
    "nfft_toeplitz_apply": (_I, [_P, _P, _P]),
    "nfft_direct": (_I, [_I, _I, _I, _I64P, _I64, _P, _P, _I, _I, _P, _P, _P]),
    "nfft_tplan_create": (_I, [ctypes.POINTER(_P), _I, _I, _I, _I64P, _I64, ctypes.POINTER(nfft_params), _P]),
    "nfft_tplan_destroy": (_I, [_P]),
    "nfft_tplan_set_stream": (_I, [_P, _P]),
    "nfft_tplan_set_nodes": (_I, [_P, _P, _I]),
    "nfft_tplan_forward": (_I, [_P, _P, _P]),
    "nfft_tplan_transpose": (_I, [_P, _P, _P]),
    "nfft_nnplan_create": (_I, [ctypes.POINTER(_P), _I, _I, _I64, _I64, ctypes.POINTER(nfft_params), _P]),
    "nfft_nnplan_destroy": (_I, [_P]),
    "nfft_nnplan_set_stream": (_I, [_P, _P]),
    "nfft_nnplan_set_nodes": (_I, [_P, _P, _P, _I]),
    "nfft_nnplan_forward": (_I, [_P, _P, _P]),
    "nfft_nnplan_adjoint": (_I, [_P, _P, _P]),
    "nfft_kernel_launch_count": (_I64, []),
    "nfft_status_string": (ctypes.c_char_p, [_I]),
    "nfft_last_error": (ctypes.c_char_p, []),
}

_lib = None


def load() -> ctypes.CDLL:
    """Load the C-ABI library (no compute happens here)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python nfft.jl_gb300/build.py` "
                "(there is no CPU fallback)")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def exported_symbols() -> list[str]:
    return sorted(SIGNATURES)
