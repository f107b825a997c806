"""satgb_sat_noalloc: the SAT entry point for callers that cannot allocate
device memory (allocator callbacks, pre-reserved device memory, loops that
must not pay for an allocation).  Its look-back scratch is a fixed array
inside libsatgb.so instead of a workspace allocated on first use.

Called through the C ABI and checked against the allocating entry point
(satgb_sat_ex) on the same input, twice in a row (the second call reuses the
array the first one left behind).  This file is collected last so that a
failure here stops a `-x` run only after every other test has run; it also
passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

from sat_gb300 import _lib
from tests.util import bits, to_dev, to_np

pytestmark = pytest.mark.gpu

TOL = {torch.float32: 1e-5, torch.float64: 1e-13}  # max |a-b| / SAT(|x|), as in test_gpu_parity
TOL_COMP = 2e-7


def _desc(x, y, mode=_lib.MODE_PLAIN, direction=_lib.FORWARD):
    from sat_gb300.api import dtype_code
    h, w = x.shape
    return _lib.satgb_sat_desc(dtype_code(x.dtype), dtype_code(y.dtype), mode, direction,
                               x.data_ptr(), x.stride(0), y.data_ptr(), y.stride(0), w, h)


def _run(fn_name, x, out_dtype, mode=_lib.MODE_PLAIN, direction=_lib.FORWARD):
    y = torch.full(x.shape, 7, dtype=torch.int32 if out_dtype == torch.uint32 else out_dtype, device=x.device)
    if out_dtype == torch.uint32:
        y = y.view(torch.uint32)
    d = _desc(x, y, mode, direction)
    stream = torch.cuda.current_stream().cuda_stream
    st = getattr(_lib.load(), fn_name)(ctypes.byref(d), stream)
    assert st == _lib.OK, (fn_name, st)
    torch.cuda.synchronize()
    return y


CASES = [
    # (name, generator kind, numpy in dtype, torch out dtype, mode, direction, shape)
    ("u8_u32", "u8", np.uint8, torch.uint32, _lib.MODE_PLAIN, _lib.FORWARD, (1000, 1500)),
    ("u8_u32_rev", "u8", np.uint8, torch.uint32, _lib.MODE_PLAIN, _lib.REVERSE, (333, 777)),
    ("f32_f32", "f32u", np.float32, torch.float32, _lib.MODE_PLAIN, _lib.FORWARD, (1024, 1024)),
    ("f32_comp", "f32log", np.float32, torch.float32, _lib.MODE_COMPENSATED, _lib.FORWARD, (700, 900)),
    ("f64_f64", "f64u", np.float64, torch.float64, _lib.MODE_PLAIN, _lib.FORWARD, (517, 613)),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_noalloc_matches_allocating_entry_point_twice(cuda, oracle, case):
    O = oracle
    name, kind, _, out_dt, mode, direction, shape = case
    a = O.gen(kind, 9000 + len(name), shape)
    x = to_dev(a)
    ref = to_np(_run("satgb_sat_ex", x, out_dt, mode, direction))
    for call in range(2):  # two calls in a row on the shared array
        got = to_np(_run("satgb_sat_noalloc", x, out_dt, mode, direction))
        if out_dt in (torch.uint32, torch.int32):
            assert np.array_equal(bits(got), bits(ref)), (name, call)
        else:
            den = O.sat_fp64(a, reverse=direction == _lib.REVERSE, absval=True)
            tol = TOL_COMP if mode == _lib.MODE_COMPENSATED else TOL[out_dt]
            err = np.abs(got.astype(np.float64) - ref.astype(np.float64))
            assert np.all(err <= 2 * tol * den), (name, call, float(np.max(err / np.maximum(den, 1e-300))))


def test_noalloc_rejects_images_beyond_its_scratch(cuda):
    x = torch.zeros((16384, 8192), dtype=torch.uint8, device="cuda")
    y = torch.zeros((16384, 8192), dtype=torch.int32, device="cuda").view(torch.uint32)
    d = _desc(x, y)
    st = _lib.load().satgb_sat_noalloc(ctypes.byref(d), torch.cuda.current_stream().cuda_stream)
    assert st == _lib.ERR_INVALID_ARG
    torch.cuda.synchronize()
    assert int(y.view(torch.int32).abs().sum().item()) == 0  # nothing was launched
