"""satgb_sat_noalloc: the SAT entry point for callers that cannot allocate
device memory (allocator callbacks, pre-reserved device memory, loops that
must not pay for an allocation).  Its look-back scratch is a fixed array
inside libsatgb.so instead of a workspace allocated on first use.

Called through the C ABI and checked against the oracle (the reference's CPU
integral image restated in C: bit-exact for integer outputs; floats against
the FP64 oracle with the tolerances of test_gpu_parity), twice in a row: the
second call reuses the array the first one left behind.  The capacity of the
array is checked at its edge: an image of exactly as many tiles as it holds
is computed correctly, one more row of tiles is rejected with a message that
names the array's size.  This file is collected last so that a failure here
stops a `-x` run only after every other test has run; it also passes on its
own in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

from sat_gb300 import _lib
from tests.util import bits, to_dev, to_np

pytestmark = pytest.mark.gpu

TOL = {torch.float32: 1e-5, torch.float64: 1e-13}  # max |S - S64| / SAT(|a|)64, as in test_gpu_parity
TOL_COMP = 2e-7
SCRATCH_BYTES = 16 << 20  # the array's size, as satgb.h states it


def _desc(x, y, mode=_lib.MODE_PLAIN, direction=_lib.FORWARD):
    from sat_gb300.api import dtype_code
    h, w = x.shape
    return _lib.satgb_sat_desc(dtype_code(x.dtype), dtype_code(y.dtype), mode, direction,
                               x.data_ptr(), x.stride(0), y.data_ptr(), y.stride(0), w, h)


def _noalloc(x, out_dtype, mode=_lib.MODE_PLAIN, direction=_lib.FORWARD):
    y = torch.full(x.shape, 7, dtype=torch.int32 if out_dtype == torch.uint32 else out_dtype, device=x.device)
    if out_dtype == torch.uint32:
        y = y.view(torch.uint32)
    d = _desc(x, y, mode, direction)
    L = _lib.load()
    before = L.satgb_launch_count()
    st = L.satgb_sat_noalloc(ctypes.byref(d), torch.cuda.current_stream().cuda_stream)
    assert st == _lib.OK, (st, L.satgb_last_error_string())
    assert L.satgb_launch_count() - before == 1  # its launch is counted like every other
    torch.cuda.synchronize()
    return y


def _check(O, a, got, out_dt, mode, direction):
    rev = direction == _lib.REVERSE
    if out_dt in (torch.uint32, torch.int32):
        npdt = np.uint32 if out_dt == torch.uint32 else np.int32
        ref = O.sat_reverse(a, npdt) if rev else O.sat_serial(a, npdt)
        assert np.array_equal(bits(got), bits(ref))
    else:
        ref = O.sat_fp64(a, reverse=rev)
        den = O.sat_fp64(a, reverse=rev, absval=True)
        tol = TOL_COMP if mode == _lib.MODE_COMPENSATED else TOL[out_dt]
        err = np.abs(got.astype(np.float64) - ref)
        assert np.all(err <= tol * den), float(np.max(err / np.maximum(den, 1e-300)))


CASES = [
    # (name, generator kind, torch out dtype, mode, direction, shape)
    ("u8_u32", "u8", torch.uint32, _lib.MODE_PLAIN, _lib.FORWARD, (1000, 1500)),
    ("u8_u32_rev", "u8", torch.uint32, _lib.MODE_PLAIN, _lib.REVERSE, (333, 777)),
    ("f32_f32", "f32u", torch.float32, _lib.MODE_PLAIN, _lib.FORWARD, (1024, 1024)),
    ("f32_comp", "f32log", torch.float32, _lib.MODE_COMPENSATED, _lib.FORWARD, (700, 900)),
    ("f64_f64", "f64u", torch.float64, _lib.MODE_PLAIN, _lib.FORWARD, (517, 613)),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_noalloc_matches_oracle_twice(cuda, oracle, case):
    name, kind, out_dt, mode, direction, shape = case
    a = oracle.gen(kind, 9000 + len(name), shape)
    x = to_dev(a)
    for call in range(2):  # two calls in a row on the shared array
        got = to_np(_noalloc(x, out_dt, mode, direction))
        _check(oracle, a, got, out_dt, mode, direction)


# The array's capacity in tiles for the three tile shapes this entry point
# uses: plain 4-byte outputs (128 x 128 tiles, one status word per row, column
# and corner), compensated f32 (64 rows x 128 columns, two words each) and f64
# (64 x 64, two words each); a 64-byte header comes first.
EDGES = [
    # (name, kind, out dtype, mode, tile width, tile height, words per value, image width)
    ("u8_u32", "u8", torch.uint32, _lib.MODE_PLAIN, 128, 128, 1, 10240),
    ("f32_comp", "f32u", torch.float32, _lib.MODE_COMPENSATED, 128, 64, 2, 384),
    ("f64_f64", "f64u", torch.float64, _lib.MODE_PLAIN, 64, 64, 2, 4096),
]


@pytest.mark.parametrize("edge", EDGES, ids=[e[0] for e in EDGES])
def test_noalloc_capacity_edge(cuda, oracle, edge):
    name, kind, out_dt, mode, tw, th, k, width = edge
    per_tile = (th + tw + 1) * k * 8
    cap = (SCRATCH_BYTES - 64) // per_tile
    ntx = width // tw
    nty = cap // ntx
    assert ntx * nty == cap, "the image width is chosen so that whole tile rows fill the array"
    # exactly the capacity: computed, and right
    a = oracle.gen(kind, 9100 + len(name), (nty * th, width))
    got = to_np(_noalloc(to_dev(a), out_dt, mode))
    _check(oracle, a, got, out_dt, mode, _lib.FORWARD)
    del got
    # one more row of tiles: rejected before any launch, with the sizes in the message
    h = nty * th + 1
    x = torch.zeros((h, width), dtype=to_dev(a[:1, :1]).dtype, device="cuda")
    y = torch.zeros((h, width), dtype=torch.int32 if out_dt == torch.uint32 else out_dt, device="cuda")
    if out_dt == torch.uint32:
        y = y.view(torch.uint32)
    L = _lib.load()
    before = L.satgb_launch_count()
    st = L.satgb_sat_noalloc(ctypes.byref(_desc(x, y, mode)), torch.cuda.current_stream().cuda_stream)
    assert st == _lib.ERR_INVALID_ARG
    assert L.satgb_launch_count() == before
    msg = L.satgb_last_error_string().decode()
    assert "satgb_sat_noalloc" in msg and str(SCRATCH_BYTES) in msg, msg
    torch.cuda.synchronize()
    assert float(y.view(torch.int32).abs().sum().item() if out_dt == torch.uint32 else y.abs().sum().item()) == 0
