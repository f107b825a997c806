"""ctypes binding of libsatgb.so (the C ABI in include/satgb.h).

The library is loaded from ``sat_gb300/_lib/`` (built in-tree by
``sat_gb300.build``).  There is no fallback: if the library is missing or
fails to load, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os
import re

from . import build as _build

# status codes (satgb_status)
OK = 0
ERR_INVALID_ARG = 1
ERR_UNSUPPORTED_TYPES = 2
ERR_MISALIGNED = 3
ERR_OVERFLOW = 4
ERR_ALLOC = 5
ERR_CUDA = 6
ERR_TIMEOUT = 7
ERR_NOT_FOUND = 8
STATUS_NAMES = {0: "SATGB_OK", 1: "SATGB_ERR_INVALID_ARG", 2: "SATGB_ERR_UNSUPPORTED_TYPES",
                3: "SATGB_ERR_MISALIGNED", 4: "SATGB_ERR_OVERFLOW", 5: "SATGB_ERR_ALLOC",
                6: "SATGB_ERR_CUDA", 7: "SATGB_ERR_TIMEOUT", 8: "SATGB_ERR_NOT_FOUND"}

# dtype codes (satgb_dtype) == the reference's DataType enum (integralImage.h:22-32)
U8, I8, U16, I16, U32, I32, F32, F64 = range(8)
# scan types == the reference's SCAN enum (integralImage.h:34-37)
KOGGE_STONE_SCAN = 0
LF_SCAN = 1
MODE_PLAIN = 0
MODE_COMPENSATED = 1
FORWARD = 0
REVERSE = 1


class SatError(RuntimeError):
    """A non-OK satgb_status, with the library's message."""

    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


class satgb_sat_desc(ctypes.Structure):
    _fields_ = [("in_t", ctypes.c_int), ("out_t", ctypes.c_int), ("mode", ctypes.c_int),
                ("direction", ctypes.c_int), ("d_in", ctypes.c_void_p), ("in_pitch", ctypes.c_int64),
                ("d_out", ctypes.c_void_p), ("out_pitch", ctypes.c_int64),
                ("width", ctypes.c_int64), ("height", ctypes.c_int64)]


class satgb_image(ctypes.Structure):
    _fields_ = [("d_in", ctypes.c_void_p), ("in_pitch", ctypes.c_int64), ("d_out", ctypes.c_void_p),
                ("out_pitch", ctypes.c_int64), ("width", ctypes.c_int64), ("height", ctypes.c_int64)]


MAX_RADII = 4


class satgb_box_desc(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int64), ("height", ctypes.c_int64), ("n_planes", ctypes.c_int64),
                ("d_sat", ctypes.c_void_p), ("sat_pitch", ctypes.c_int64), ("sat_plane_stride", ctypes.c_int64),
                ("n_radii", ctypes.c_int), ("radius", ctypes.c_int * MAX_RADII),
                ("d_box", ctypes.c_void_p * MAX_RADII), ("box_pitch", ctypes.c_int64),
                ("box_plane_stride", ctypes.c_int64)]


_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_ST = ctypes.c_int
_ALLOC_FN = ctypes.CFUNCTYPE(ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p)
_FREE_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_void_p)

# name -> (restype, argtypes)
SIGNATURES = {
    "satgb_scanrow_brlt": (_ST, [_I, _I, _I, _P, _I64, _P, _I64, _I64, _I64, _P]),
    "satgb_brlt_scanrow": (_ST, [_I, _I, _I, _P, _I64, _P, _I64, _I64, _I64, _P]),
    "satgb_scanrowcolumn": (_ST, [_I, _I, _I, _P, _I64, _P, _I64, _I64, _I64, _P]),
    "satgb_sat_ex": (_ST, [ctypes.POINTER(satgb_sat_desc), _P]),
    "satgb_sat_noalloc": (_ST, [ctypes.POINTER(satgb_sat_desc), _P]),
    "satgb_batch_plan_create": (_ST, [ctypes.POINTER(_P), _I, _I, _I, _I, ctypes.POINTER(satgb_image), _I64, _P]),
    "satgb_batch_plan_exec": (_ST, [_P, _P]),
    "satgb_batch_plan_launch": (_ST, [_P, _P]),
    "satgb_batch_plan_destroy": (_ST, [_P]),
    "satgb_batch_plan_info": (_ST, [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I)]),
    "satgb_batch_plan_check": (_ST, [_P, _P]),
    "satgb_batch_plan_classes": (_ST, [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64), ctypes.POINTER(_I)]),
    "satgb_batch_plan_autotune": (_ST, [_P, _P, ctypes.POINTER(_I)]),
    "satgb_autotune": (_ST, [_I, _I, _I, _P, _I64, _P, _I64, _I64, _I64, _P, ctypes.POINTER(_I)]),
    "satgb_num_configs": (_I, []),
    "satgb_config_name": (ctypes.c_char_p, [_I]),
    "satgb_set_config": (_ST, [_I]),
    "satgb_stream_check": (_ST, [_P]),
    "satgb_last_error_string": (ctypes.c_char_p, []),
    "satgb_release": (_ST, []),
    "satgb_reserve": (_ST, [_I64, _I64, _P]),
    "satgb_set_allocator": (_ST, [_ALLOC_FN, _FREE_FN, _P]),
    "satgb_set_wait_limit_us": (_ST, [_I64]),
    "satgb_launch_count": (_I64, []),
    "satgb_debug_stall_tile": (_ST, [_I64]),
    "satgb_version": (_I, []),
    "satgb_sat_planes": (_ST, [ctypes.POINTER(satgb_sat_desc), _I64, _I64, _I64, _P]),
    "satgb_scan_rows": (_ST, [_I, _I, _P, _I64, _P, _I64, _I64, _I64, _P]),
    "satgb_scan_rows_transposed": (_ST, [_I, _I, _P, _I64, _P, _I64, _I64, _I64, _P]),
    "satgb_scan_cols": (_ST, [_I, _I, _P, _I64, _P, _I64, _I64, _I64, _P]),
    "satgb_box_filter_fwd": (_ST, [ctypes.POINTER(satgb_box_desc), _P]),
    "satgb_box_filter_bwd": (_ST, [ctypes.POINTER(satgb_box_desc), _P]),
    "satgb_box_filter_bwd_x": (_ST, [ctypes.POINTER(satgb_box_desc), _P, _I64, _I64, _P]),
}

_lib = None


def header_symbols() -> list:
    """Every function declared in include/satgb.h."""
    hdr = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "satgb.h")
    text = open(hdr).read()
    return sorted(set(re.findall(r"\b(satgb_[a-z0-9_]+)\s*\(", text)) - {"satgb_alloc_fn", "satgb_free_fn"})


def load(path: str = None) -> ctypes.CDLL:
    """Loads libsatgb.so (no GPU needed to load it)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or _build.lib_path()
    if not os.path.isfile(path):
        raise ImportError(f"libsatgb.so is not built ({path}); run `python -m sat_gb300.build`")
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name, None)
        if f is None:
            continue
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(status: int) -> None:
    if status != OK:
        msg = load().satgb_last_error_string()
        raise SatError(status, msg.decode() if msg else "")


def launch_count() -> int:
    return int(load().satgb_launch_count())
