"""CPU oracle for the SAT hot path -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module, and only as the checker (or as the timed CPU baseline), never as
the thing measured or shipped.  The product (``sat_gb300``) never imports it.

Three layers:

* ``liboracle.so`` built from ``oracle/sat_oracle.c``: a C restatement of the
  reference's ``IntegralImageSerial`` / ``IntegralImageParallel``
  (pengdada/SAT integralImage/integralImage.h:105-124 and :129-146), a
  double-double FP64 SAT (forward and reverse), error statistics and the
  splitmix64 input generator.
* ``libref_sat.so`` (optional, ``oracle/_ref/``): the reference's own CPU code
  compiled from its header by ``make -C oracle ref``; present only where the
  reference checkout is (never on the GPU host).
* Pure-numpy restatements for small cases (``sat_serial_np``) that pin the C
  restatement from a second, independent implementation.

Pitches are in elements, as in the reference (cudaLib.cuh:178-180).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")
REF_LIB_PATH = os.path.join(REF_DIR, "libref_sat.so")
# The reference checkout's integralImage/ directory, where one is present,
# is named by the SATGB_REF_DIR environment variable (no default): without it
# only the restatement is built, and the tests that need the reference's own
# code skip.
REF_DIR_ENV = "SATGB_REF_DIR"

# dtype-pair name -> (numpy in dtype, numpy out dtype)
PAIRS = {
    "u8_u32": (np.uint8, np.uint32),
    "u8_f32": (np.uint8, np.float32),
    "u8_f64": (np.uint8, np.float64),
    "i8_i32": (np.int8, np.int32),
    "i8_f32": (np.int8, np.float32),
    "i8_f64": (np.int8, np.float64),
    "i32_i32": (np.int32, np.int32),
    "i32_f64": (np.int32, np.float64),
    "u32_u32": (np.uint32, np.uint32),
    "f32_f32": (np.float32, np.float32),
    "f32_f64": (np.float32, np.float64),
    "f64_f64": (np.float64, np.float64),
}
_DD_IN = {np.uint8: "u8", np.int8: "i8", np.uint32: "u32", np.int32: "i32",
          np.float32: "f32", np.float64: "f64"}
_NP_NAME = {np.dtype(k).name: v for k, v in _DD_IN.items()}


def pair_name(in_dtype, out_dtype) -> str:
    a = _NP_NAME[np.dtype(in_dtype).name]
    b = _NP_NAME[np.dtype(out_dtype).name]
    return f"{a}_{b}"


# ----------------------------------------------------------------------------
# building and loading
# ----------------------------------------------------------------------------

def build(with_ref: Optional[bool] = None, quiet: bool = True) -> None:
    """Compile liboracle.so; also the reference's own CPU code into _ref/ when
    SATGB_REF_DIR names the reference checkout (``with_ref=None`` means "if
    it does")."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.check_call(["make", "-s", "-C", HERE, "all"], stdout=out)
    ref_src = os.environ.get(REF_DIR_ENV, "")
    present = bool(ref_src) and os.path.isfile(os.path.join(ref_src, "integralImage.h"))
    if with_ref is None:
        with_ref = present
    if with_ref:
        if not present:
            raise RuntimeError(f"{REF_DIR_ENV} must name the reference's integralImage/ directory")
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", f"REF_DIR={ref_src}"],
                              stdout=out, stderr=subprocess.DEVNULL if quiet else None)


_lib = None
_ref = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.isfile(LIB_PATH):
            build(with_ref=False)
        _lib = ctypes.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


def ref_lib() -> Optional[ctypes.CDLL]:
    """The reference's own CPU integral image, or None where it was not built."""
    global _ref
    if _ref is None and os.path.isfile(REF_LIB_PATH):
        _ref = ctypes.CDLL(REF_LIB_PATH)
    return _ref


_P = ctypes.c_void_p
_I64 = ctypes.c_int64


def _declare(L: ctypes.CDLL) -> None:
    for name in PAIRS:
        for fname in (f"oracle_sat_serial_{name}", f"oracle_sat_reverse_{name}", f"oracle_scan_rows_{name}",
                      f"oracle_scan_cols_{name}"):
            f = getattr(L, fname)
            f.argtypes = [_P, _I64, _P, _I64, _I64, _I64]
            f.restype = None
        f = getattr(L, f"oracle_sat_parallel_{name}")
        f.argtypes = [_P, _I64, _P, _I64, _I64, _I64, ctypes.c_int]
        f.restype = None
    for t in ("u8", "i8", "u32", "i32", "f32", "f64"):
        f = getattr(L, f"oracle_sat_dd_{t}")
        f.argtypes = [_P, _I64, _P, _I64, _I64, _I64, ctypes.c_int, ctypes.c_int, _P]
        f.restype = ctypes.c_int
    for t in ("f32", "f64"):
        f = getattr(L, f"oracle_err_stats_{t}")
        f.argtypes = [_P, _I64, _P, _P, _I64, _I64, _P]
        f.restype = None
    for g in ("u8", "u32", "f32_uniform", "f64_uniform"):
        f = getattr(L, f"oracle_gen_{g}")
        f.argtypes = [ctypes.c_uint64, _I64, _P]
        f.restype = None
    L.oracle_num_threads.restype = ctypes.c_int


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def _pitch(a: np.ndarray) -> int:
    assert a.ndim == 2
    if a.size == 0:
        return max(a.shape[1], 1)
    assert (a.shape[1] == 1 or a.strides[1] == a.itemsize) and a.strides[0] % a.itemsize == 0
    return a.strides[0] // a.itemsize if a.shape[0] > 1 else a.shape[1]


# ----------------------------------------------------------------------------
# the reference's algorithm, restated
# ----------------------------------------------------------------------------

def sat_serial(a: np.ndarray, out_dtype) -> np.ndarray:
    """IntegralImageSerial<TSrc,TDst> (integralImage.h:105-124), C restatement."""
    h, w = a.shape
    name = pair_name(a.dtype, out_dtype)
    out = np.zeros((h, w), dtype=out_dtype)
    getattr(lib(), f"oracle_sat_serial_{name}")(_ptr(a), _pitch(a), _ptr(out), w, w, h)
    return out


def sat_parallel(a: np.ndarray, out_dtype, nthreads: int = 0) -> np.ndarray:
    """IntegralImageParallel (integralImage.h:129-146), C + OpenMP restatement."""
    h, w = a.shape
    name = pair_name(a.dtype, out_dtype)
    out = np.empty((h, w), dtype=out_dtype)
    n = nthreads or lib().oracle_num_threads()
    getattr(lib(), f"oracle_sat_parallel_{name}")(_ptr(a), _pitch(a), _ptr(out), w, w, h, n)
    return out


def scan_rows(a: np.ndarray, out_dtype) -> np.ndarray:
    """Row-only scan: IntegralRow (integralImage.h:74-82) on every row, as
    IncrementScanX computes it; C restatement in the output type."""
    h, w = a.shape
    out = np.zeros((h, w), dtype=out_dtype)
    getattr(lib(), f"oracle_scan_rows_{pair_name(a.dtype, out_dtype)}")(_ptr(a), _pitch(a), _ptr(out), w, w, h)
    return out


def scan_cols(a: np.ndarray, out_dtype) -> np.ndarray:
    """Column-only scan: IntegralStride (integralImage.h:90-101) with the row
    stride, on every column, as IncrementScanY computes it."""
    h, w = a.shape
    out = np.zeros((h, w), dtype=out_dtype)
    getattr(lib(), f"oracle_scan_cols_{pair_name(a.dtype, out_dtype)}")(_ptr(a), _pitch(a), _ptr(out), w, w, h)
    return out


def sat_reverse(a: np.ndarray, out_dtype) -> np.ndarray:
    """Suffix SAT R(y,x) = sum_{j>=y,i>=x} a(j,i), serial, in the output type."""
    h, w = a.shape
    name = pair_name(a.dtype, out_dtype)
    out = np.zeros((h, w), dtype=out_dtype)
    getattr(lib(), f"oracle_sat_reverse_{name}")(_ptr(a), _pitch(a), _ptr(out), w, w, h)
    return out


def sat_fp64(a: np.ndarray, reverse: bool = False, absval: bool = False) -> np.ndarray:
    """FP64 oracle: SAT (or suffix SAT, or SAT of |a|) in double-double,
    rounded once to double."""
    h, w = a.shape
    t = _NP_NAME[a.dtype.name]
    out = np.empty((h, w), dtype=np.float64)
    scratch = np.empty(2 * max(w, 1), dtype=np.float64)
    getattr(lib(), f"oracle_sat_dd_{t}")(_ptr(a), _pitch(a), _ptr(out), w, w, h,
                                          int(reverse), int(absval), _ptr(scratch))
    return out


def err_stats(s: np.ndarray, ref64: np.ndarray, refabs64: Optional[np.ndarray] = None) -> dict:
    """max/mean of |S-S64|/|S64| and of |S-S64|/SAT(|a|)64."""
    h, w = ref64.shape
    res = np.zeros(4, dtype=np.float64)
    t = "f32" if s.dtype == np.float32 else "f64"
    r = np.ascontiguousarray(ref64)
    ra = None if refabs64 is None else np.ascontiguousarray(refabs64)
    getattr(lib(), f"oracle_err_stats_{t}")(_ptr(s), _pitch(s), _ptr(r),
                                             None if ra is None else _ptr(ra), w, h, _ptr(res))
    return {"max_rel": res[0], "mean_rel": res[1], "max_rel_abs": res[2], "mean_rel_abs": res[3]}


def ref_serial(a: np.ndarray, out_dtype) -> Optional[np.ndarray]:
    """The reference's own IntegralImageSerial, or None where it is not built."""
    R = ref_lib()
    if R is None:
        return None
    h, w = a.shape
    a = np.ascontiguousarray(a)
    out = np.zeros((h, w), dtype=out_dtype)
    f = getattr(R, f"ref_serial_{pair_name(a.dtype, out_dtype)}")
    f.argtypes = [_P, _P, ctypes.c_int, ctypes.c_int]
    f.restype = None
    f(_ptr(a), _ptr(out), w, h)
    return out


def _ref_scan(kind: str, a: np.ndarray, out_dtype) -> Optional[np.ndarray]:
    R = ref_lib()
    if R is None:
        return None
    h, w = a.shape
    a = np.ascontiguousarray(a)
    name = pair_name(a.dtype, out_dtype)
    if kind == "allrow_t":
        tmp = np.zeros((h, w), dtype=out_dtype)
        out = np.zeros((w, h), dtype=out_dtype)
        f = getattr(R, f"ref_allrow_t_{name}")
        f.argtypes = [_P, _P, _P, ctypes.c_int, ctypes.c_int]
        f.restype = None
        f(_ptr(a), _ptr(tmp), _ptr(out), w, h)
        return out
    out = np.zeros((h, w), dtype=out_dtype)
    f = getattr(R, f"ref_{kind}_{name}")
    f.argtypes = [_P, _P, ctypes.c_int, ctypes.c_int]
    f.restype = None
    f(_ptr(a), _ptr(out), w, h)
    return out


def ref_scan_rows(a: np.ndarray, out_dtype) -> Optional[np.ndarray]:
    """The reference's own IntegralImageAllRow, or None where it is not built."""
    return _ref_scan("allrow", a, out_dtype)


def ref_scan_rows_transposed(a: np.ndarray, out_dtype) -> Optional[np.ndarray]:
    """The reference's IntegralImageAllRow followed by its Transpose (the check
    of SerielScan::TestX), a (W, H) array, or None where it is not built."""
    return _ref_scan("allrow_t", a, out_dtype)


def ref_scan_cols(a: np.ndarray, out_dtype) -> Optional[np.ndarray]:
    """The reference's own IntegralStride down every column, or None."""
    return _ref_scan("colscan", a, out_dtype)


def ref_parallel(a: np.ndarray) -> Optional[np.ndarray]:
    """The reference's own IntegralImageParallel<T,T> (matching types only)."""
    R = ref_lib()
    if R is None:
        return None
    h, w = a.shape
    a = np.ascontiguousarray(a)
    out = np.zeros((h, w), dtype=a.dtype)
    f = getattr(R, f"ref_parallel_{pair_name(a.dtype, a.dtype)}")
    f.argtypes = [_P, _P, ctypes.c_int, ctypes.c_int]
    f.restype = None
    f(_ptr(a), _ptr(out), w, h)
    return out


# ----------------------------------------------------------------------------
# pure-numpy restatement for small cases
# ----------------------------------------------------------------------------

def sat_serial_np(a: np.ndarray, out_dtype) -> np.ndarray:
    """Loop-for-loop numpy restatement of IntegralImageSerial for small cases:
    out[0] = running row sum; out[y] = out[y-1] + running row sum of row y,
    in the output type (integer outputs wrap mod 2^32)."""
    h, w = a.shape
    out_dtype = np.dtype(out_dtype)
    acc = np.uint32 if out_dtype.kind in "iu" else out_dtype.type
    out = np.zeros((h, w), dtype=acc)
    with np.errstate(over="ignore"):
        for y in range(h):
            row = a[y].astype(np.int64).astype(acc) if out_dtype.kind in "iu" else a[y].astype(acc)
            s = acc(0)
            for x in range(w):
                s = acc(s + row[x])
                out[y, x] = s if y == 0 else acc(out[y - 1, x] + s)
    return out.view(out_dtype) if out_dtype.kind in "iu" else out


# ----------------------------------------------------------------------------
# inputs: splitmix64 counter-based generator (same as oracle_gen_* in C)
# ----------------------------------------------------------------------------
_GAMMA = np.uint64(0x9E3779B97F4A7C15)


def _mix(z: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def _stream(seed: int, n: int) -> np.ndarray:
    key = _mix(np.array([np.uint64(seed) ^ np.uint64(0x5A7A5A7A5A7A5A7A)], dtype=np.uint64))[0]
    with np.errstate(over="ignore"):
        i = np.arange(1, n + 1, dtype=np.uint64)
        return _mix(key + i * _GAMMA)


def gen(kind: str, seed: int, shape, use_c: bool = True) -> np.ndarray:
    """Seeded synthetic image.

    kinds: "u8" uniform 0-255; "u32" uniform 32-bit; "i8" uniform -128..127;
    "i32" uniform signed 32-bit; "f32u" uniform [0,1) (24 bits, exact in f32);
    "f64u" uniform [0,1) (53 bits); "f32log" magnitude 10^U(-3,3) with random
    sign; "f32n" / "f64n" standard normal (Box-Muller); "bin" 0/1 values (the
    reference's own rand()%2 inputs, ScanRow-BRLT.cu:207).
    """
    h, w = shape
    n = h * w
    L = lib() if use_c else None
    if kind == "u8" and L is not None:
        out = np.empty(n, dtype=np.uint8)
        L.oracle_gen_u8(seed, n, _ptr(out))
        return out.reshape(h, w)
    if kind == "u32" and L is not None:
        out = np.empty(n, dtype=np.uint32)
        L.oracle_gen_u32(seed, n, _ptr(out))
        return out.reshape(h, w)
    if kind == "f32u" and L is not None:
        out = np.empty(n, dtype=np.float32)
        L.oracle_gen_f32_uniform(seed, n, _ptr(out))
        return out.reshape(h, w)
    if kind == "f64u" and L is not None:
        out = np.empty(n, dtype=np.float64)
        L.oracle_gen_f64_uniform(seed, n, _ptr(out))
        return out.reshape(h, w)
    z = _stream(seed, n)
    if kind == "u8":
        out = (z >> np.uint64(56)).astype(np.uint8)
    elif kind == "u32":
        out = (z >> np.uint64(32)).astype(np.uint32)
    elif kind == "i8":
        out = (z >> np.uint64(56)).astype(np.uint8).view(np.int8)
    elif kind == "i32":
        out = (z >> np.uint64(32)).astype(np.uint32).view(np.int32)
    elif kind == "bin":
        out = (z >> np.uint64(63)).astype(np.uint8)
    elif kind == "f32u":
        out = ((z >> np.uint64(40)).astype(np.float32) * np.float32(1.0 / 16777216.0))
    elif kind == "f64u":
        out = (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    elif kind == "f32log":
        u = (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        sign = np.where((z & np.uint64(1)) == 1, -1.0, 1.0)
        out = (sign * np.power(10.0, -3.0 + 6.0 * u)).astype(np.float32)
    elif kind in ("f32n", "f64n"):
        z2 = _stream(seed ^ 0x1234567, n)
        u1 = ((z >> np.uint64(11)).astype(np.float64) + 1.0) * (1.0 / 9007199254740992.0)
        u2 = (z2 >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        g = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)
        out = g.astype(np.float32 if kind == "f32n" else np.float64)
    else:
        raise ValueError(kind)
    return out.reshape(h, w)
