"""Parity of the CUDA path (through the C ABI) with the oracle.

Integer outputs must be bit-exact against the reference's CPU integral image
(golden vectors made by running it, and the C restatement for other inputs),
including the mod-2^32 wrap.  Float outputs are compared with the FP64
oracle with the tolerances below, stated relative to SAT(|a|) computed in
FP64 (the denominator that stays meaningful under cancellation):

  plain f32       max |S - S64| / SAT(|a|)64  <= 1e-5
  compensated f32 max |S - S64| / SAT(|a|)64  <= 2e-7   (one final rounding)
  f64             max |S - S64| / SAT(|a|)64  <= 1e-13
"""
import hashlib

import numpy as np
import pytest
import torch

import sat_gb300
from sat_gb300 import _lib
from tests.util import bits, empty_pitched, to_dev, to_np

pytestmark = pytest.mark.gpu

TOL = {np.dtype(np.float32): 1e-5, np.dtype(np.float64): 1e-13}
TOL_COMP = 2e-7
ALGOS = [sat_gb300.scanrow_brlt, sat_gb300.brlt_scanrow, sat_gb300.scanrowcolumn]


def _check_float(oracle, a, s, tol, reverse=False):
    ref = oracle.sat_fp64(a, reverse=reverse)
    den = oracle.sat_fp64(a, reverse=reverse, absval=True)
    err = np.abs(s.astype(np.float64) - ref)
    mask = den > 0
    worst = float(np.max(err[mask] / den[mask])) if mask.any() else 0.0
    assert np.all(err[~mask] == 0)
    assert worst <= tol, worst
    return worst


def _check(oracle, a, out_np, out_dtype, tol=None, reverse=False):
    out_dtype = np.dtype(out_dtype)
    if out_dtype.kind in "iu":
        ref = oracle.sat_reverse(a, out_dtype) if reverse else oracle.sat_serial(a, out_dtype)
        assert np.array_equal(bits(out_np), bits(ref))
    else:
        _check_float(oracle, a, out_np, tol or TOL[out_dtype], reverse)


def test_golden_small_all_entry_points(cuda, oracle, golden):
    z, meta = golden
    for case in meta["small"]:
        a = z[case["key"] + "__in"]
        r = z[case["key"] + "__out"]
        x = to_dev(a)
        for fn in ALGOS:
            for scan in (sat_gb300.KOGGE_STONE_SCAN, sat_gb300.LF_SCAN):
                out = to_np(fn(x, torch.float32 if r.dtype == np.float32 else
                               {np.dtype(np.uint32): torch.uint32, np.dtype(np.int32): torch.int32,
                                np.dtype(np.float64): torch.float64}[r.dtype], scan_type=scan))
                if r.dtype.kind in "iu":
                    assert np.array_equal(bits(out), bits(r)), (case["key"], fn.__name__)
                else:
                    _check_float(oracle, a, out, TOL[r.dtype])
                    _check_float(oracle, a, r, TOL[r.dtype])  # the reference itself meets the same bound


def test_reference_size_1024_digests(cuda, oracle, golden):
    """The reference's smallest benchmark size (1024 x 1024, ScanRow-BRLT.cu:272-273)
    through all three entry points."""
    _, meta = golden
    for case in meta["big"]:
        ti, to = oracle.PAIRS[case["pair"]]
        a = oracle.gen(case["kind"], case["seed"], (case["h"], case["w"])).astype(ti)
        assert hashlib.sha256(a.tobytes()).hexdigest() == case["in_sha256"]
        x = to_dev(a)
        for fn in ALGOS:
            out = to_np(fn(x, {np.dtype(np.uint32): torch.uint32, np.dtype(np.float32): torch.float32,
                               np.dtype(np.float64): torch.float64}[np.dtype(to)]))
            if np.dtype(to).kind in "iu":
                assert hashlib.sha256(out.tobytes()).hexdigest() == case["out_sha256"], (case["key"], fn.__name__)
            else:
                _check_float(oracle, a, out, TOL[np.dtype(to)])


PAIR_KINDS = {np.uint8: "u8", np.int8: "i8", np.int32: "i32", np.uint32: "u32",
              np.float32: "f32u", np.float64: "f64u"}
SHAPES = [(1, 1), (1, 700), (700, 1), (2, 3), (63, 127), (64, 128), (65, 129), (127, 255),
          (129, 257), (300, 1000), (1000, 300), (517, 769)]


@pytest.mark.parametrize("cfg", [0, 1, 2, 3, 4, 5, 6])
def test_all_pairs_all_configs(cuda, oracle, cfg):
    sat_gb300.set_config(cfg)
    try:
        for name, (ti, to) in oracle.PAIRS.items():
            for i, shape in enumerate(SHAPES):
                a = oracle.gen(PAIR_KINDS[ti], 1000 + i, shape)
                out = sat_gb300.sat(to_dev(a), {np.uint32: torch.uint32, np.int32: torch.int32,
                                                np.float32: torch.float32, np.float64: torch.float64}[to])
                _check(oracle, a, to_np(out), to)
    finally:
        sat_gb300.set_config(-1)


@pytest.mark.parametrize("cfg", [0, 1, 2, 3, 4, 5, 6])
def test_reverse_all_configs(cuda, oracle, cfg):
    sat_gb300.set_config(cfg)
    try:
        for name in ("u8_u32", "i32_i32", "f32_f32", "f64_f64", "u8_f64"):
            ti, to = oracle.PAIRS[name]
            for i, shape in enumerate(SHAPES):
                a = oracle.gen(PAIR_KINDS[ti], 2000 + i, shape)
                out = sat_gb300.sat(to_dev(a), {np.uint32: torch.uint32, np.int32: torch.int32,
                                                np.float32: torch.float32, np.float64: torch.float64}[to],
                                    reverse=True)
                _check(oracle, a, to_np(out), to, reverse=True)
    finally:
        sat_gb300.set_config(-1)


def test_pitched_unaligned_and_inplace(cuda, oracle):
    # pitch > width with vector-aligned rows
    a = oracle.gen("u8", 7, (333, 555))
    src = empty_pitched(333, 555, 640, torch.uint8)
    src.copy_(to_dev(a))
    dst = empty_pitched(333, 555, 600, torch.uint32, fill=-1)
    sat_gb300.scanrowcolumn(src, torch.uint32, out=dst)
    assert np.array_equal(to_np(dst), oracle.sat_serial(a, np.uint32))
    # odd pitch: rows not 4-byte aligned -> scalar loads
    src2 = empty_pitched(333, 555, 557, torch.uint8)
    src2.copy_(to_dev(a))
    dst2 = empty_pitched(333, 555, 559, torch.uint32)
    sat_gb300.scanrow_brlt(src2, torch.uint32, out=dst2)
    assert np.array_equal(to_np(dst2), oracle.sat_serial(a, np.uint32))
    # base pointer offset by one element (misaligned for vectors, aligned for elements)
    big = torch.zeros(1 + 200 * 300, dtype=torch.uint8, device="cuda")
    view = big[1:].view(200, 300)
    b = oracle.gen("u8", 8, (200, 300))
    view.copy_(to_dev(b))
    out = sat_gb300.brlt_scanrow(view, torch.uint32)
    assert np.array_equal(to_np(out), oracle.sat_serial(b, np.uint32))
    # the padding between rows is never written
    pad = dst.as_strided((333, 45), (600, 1), dst.storage_offset() + 555)
    assert np.all(to_np(pad) == np.uint32(0xFFFFFFFF))
    # in place, f32 -> f32 on one buffer
    f = oracle.gen("f32u", 9, (400, 700))
    x = to_dev(f)
    sat_gb300.sat(x, torch.float32, out=x)
    _check(oracle, f, to_np(x), np.float32)


@pytest.mark.parametrize("pair", ["u8_u32", "u8_f64", "f32_f32", "f64_f64", "i8_i32"])
def test_aligned_pitch_ragged_width(cuda, oracle, pair):
    """16-byte aligned pitches with widths that end mid-chunk: the tensor maps
    cover the whole 16-byte chunks and the row tails go by plain accesses.
    The row padding (sentinel-filled) must stay untouched, forward and reverse."""
    ti, to = oracle.PAIRS[pair]
    ti, to = np.dtype(ti), np.dtype(to)
    kind = {"u1": "u8", "i1": "i8", "f4": "f32u", "f8": "f64u"}[ti.str[1:]]
    tin = {np.dtype(np.uint8): torch.uint8, np.dtype(np.int8): torch.int8,
           np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64}[ti]
    tout = {np.dtype(np.uint32): torch.uint32, np.dtype(np.int32): torch.int32,
            np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64}[to]
    for h, w in [(70, 17), (131, 555), (66, 1001), (40, 3), (257, 129)]:
        a = oracle.gen(kind, 40 + w, (h, w)).astype(ti)
        pin = -(-w * ti.itemsize // 64) * 64 // ti.itemsize + 16 // ti.itemsize
        pout = -(-w * to.itemsize // 64) * 64 // to.itemsize + 16 // to.itemsize
        src = empty_pitched(h, w, pin, tin)
        src.copy_(to_dev(a))
        fill = -1 if to.kind in "iu" else float("nan")
        for rev in (False, True):
            dst = empty_pitched(h, w, pout, tout, fill=fill)
            sat_gb300.sat(src, tout, reverse=rev, out=dst)
            _check(oracle, a, to_np(dst), to, reverse=rev)
            pad = dst.as_strided((h, pout - w), (pout, 1), dst.storage_offset() + w)
            padn = to_np(pad)
            if to.kind in "iu":
                assert np.all(bits(padn) == 0xFF), (h, w, rev)
            else:
                assert np.all(np.isnan(padn)), (h, w, rev)


def test_back_to_back_calls_reuse_workspace(cuda, oracle):
    rng = np.random.default_rng(0)
    outs = []
    for i in range(40):
        h, w = int(rng.integers(1, 900)), int(rng.integers(1, 900))
        a = oracle.gen("u8", 3000 + i, (h, w))
        outs.append((a, sat_gb300.scanrow_brlt(to_dev(a), torch.uint32)))
    sat_gb300.stream_check()
    for a, o in outs:
        assert np.array_equal(to_np(o), oracle.sat_serial(a, np.uint32))


def test_other_stream(cuda, oracle):
    s = torch.cuda.Stream()
    a = oracle.gen("u8", 44, (1500, 1300))
    x = to_dev(a)
    torch.cuda.synchronize()
    with torch.cuda.stream(s):
        out = sat_gb300.scanrowcolumn(x, torch.uint32)
    s.synchronize()
    sat_gb300.stream_check(s)
    assert np.array_equal(to_np(out), oracle.sat_serial(a, np.uint32))


@pytest.mark.parametrize("kind", ["f32u", "f32log"])
def test_compensated_f32(cuda, oracle, kind):
    a = oracle.gen(kind, 55, (2048, 2048))
    x = to_dev(a)
    plain = to_np(sat_gb300.sat(x, torch.float32))
    comp = to_np(sat_gb300.sat(x, torch.float32, mode="compensated"))
    ref = oracle.sat_fp64(a)
    den = oracle.sat_fp64(a, absval=True)
    e_plain = oracle.err_stats(plain, ref, den)
    e_comp = oracle.err_stats(comp, ref, den)
    assert e_plain["max_rel_abs"] <= 1e-5, e_plain
    assert e_comp["max_rel_abs"] <= TOL_COMP, e_comp
    if kind == "f32u":
        assert e_comp["max_rel"] <= 1e-6, e_comp
    # compensated reverse too
    rc = to_np(sat_gb300.sat(x, torch.float32, mode="compensated", reverse=True))
    e_rev = oracle.err_stats(rc, oracle.sat_fp64(a, reverse=True), oracle.sat_fp64(a, reverse=True, absval=True))
    assert e_rev["max_rel_abs"] <= TOL_COMP, e_rev


@pytest.mark.parametrize("kind", ["f32u", "f32log"])
def test_compensated_register_tiles_forward_and_reverse(cuda, oracle, kind):
    """Configuration 3 (the register-resident 128-row tiles, the default for
    large compensated images) forced on every edge shape and at 2048^2,
    forward and reverse: the reverse compensated SAT is the backward of the
    compensated autograd SAT."""
    sat_gb300.set_config(3)
    try:
        for i, shape in enumerate(SHAPES + [(2048, 2048)]):
            a = oracle.gen(kind, 6000 + i, shape)
            x = to_dev(a)
            for rev in (False, True):
                out = to_np(sat_gb300.sat(x, torch.float32, mode="compensated", reverse=rev))
                _check_float(oracle, a, out, TOL_COMP, reverse=rev)
    finally:
        sat_gb300.set_config(-1)


def test_compensated_u8_and_i8_inputs(cuda, oracle):
    for kind, dt in (("u8", np.uint8), ("i8", np.int8)):
        a = oracle.gen(kind, 66, (1000, 1500))
        comp = to_np(sat_gb300.sat(to_dev(a), torch.float32, mode="compensated"))
        exact = a.astype(np.int64).cumsum(0).cumsum(1)
        # integer-valued sums: compensated f32 is the exact sum rounded once
        assert np.array_equal(comp, exact.astype(np.float32))


def test_batch_plan_uneven(cuda, oracle):
    rng = np.random.default_rng(5)
    ins, outs, arrs = [], [], []
    for i in range(48):
        h = int(np.exp(rng.uniform(np.log(1), np.log(700))))
        w = int(np.exp(rng.uniform(np.log(1), np.log(700))))
        a = oracle.gen("u8", 4000 + i, (h, w))
        arrs.append(a)
        ins.append(to_dev(a))
        outs.append(torch.empty((h, w), dtype=torch.uint32, device="cuda"))
    plan = sat_gb300.BatchPlan(ins, outs)
    assert plan.info()["n_tiles"] > 48
    for rep in range(3):
        for o in outs:
            o.fill_(0)
        (plan.exec if rep != 1 else plan.launch)()
        plan.check()
        for a, o in zip(arrs, outs):
            assert np.array_equal(to_np(o), oracle.sat_serial(a, np.uint32))
    plan.close()


def test_batch_plan_stages_unaligned_inputs_each_exec(cuda, oracle):
    """Inputs whose rows TMA cannot address (packed rows of odd widths, an
    offset base) are copied into the plan's padded staging rows at every
    execution: after the caller changes its inputs in place, the next exec
    reads the new values.  Mixed with 16-byte pitched images and rows shorter
    than 16 bytes, which are not staged."""
    rng = np.random.default_rng(9)
    ins, outs, views = [], [], []
    for i in range(24):
        h, w = int(rng.integers(1, 400)), int(rng.integers(1, 900))
        if i % 3 == 0:  # 16-byte pitched rows: TMA reads them in place
            x = empty_pitched(h, w, (w + 15) // 16 * 16, torch.uint8)
        elif i % 3 == 1:  # packed rows, one byte past a 16-byte boundary
            x = torch.empty(h * w + 1, dtype=torch.uint8, device=cuda)[1:].view(h, w)
        else:  # packed rows
            x = torch.empty((h, w), dtype=torch.uint8, device=cuda)
        ins.append(x)
        outs.append(torch.empty((h, w), dtype=torch.uint32, device=cuda))
    plan = sat_gb300.BatchPlan(ins, outs)
    for rep in range(2):
        arrs = [oracle.gen("u8", 6000 + 100 * rep + i, tuple(x.shape)) for i, x in enumerate(ins)]
        for x, a in zip(ins, arrs):
            x.copy_(to_dev(a))
        plan.exec()
        plan.check()
        for a, o in zip(arrs, outs):
            assert np.array_equal(to_np(o), oracle.sat_serial(a, np.uint32)), rep
    plan.close()


@pytest.mark.parametrize("layout", ["packed", "offset"])
def test_single_image_staged_input(cuda, oracle, layout):
    """A single image of 1-byte inputs, at least 2^22 pixels, whose rows TMA
    cannot address (packed rows of an odd width, or a base one byte past a
    16-byte boundary) is copied into padded rows of the workspace by one more
    launch before the tile kernel: bit-exact against the oracle, both
    directions, and again after the input changes in place."""
    h, w = 2049, 2051
    n = h * w + 1
    for rev in (False, True):
        for rep in range(2):
            a = oracle.gen("u8", 7100 + 10 * rep + rev, (h, w))
            if layout == "packed":
                x = to_dev(a)
            else:
                x = torch.empty(n + 16, dtype=torch.uint8, device=cuda)[1:1 + h * w].view(h, w)
                x.copy_(to_dev(a))
            before = sat_gb300.launch_count()
            out = sat_gb300.sat(x, torch.uint32, reverse=rev)
            assert sat_gb300.launch_count() - before == 2  # the staging copy and the SAT
            ref = oracle.sat_reverse(a, np.uint32) if rev else oracle.sat_serial(a, np.uint32)
            assert np.array_equal(to_np(out), ref), (layout, rev, rep)


def test_reserve_then_capture_staged_call(cuda, oracle):
    """satgb_reserve sizes the stream's workspace for the staging rows too: a
    staged single-image call (packed u8 rows, 2049 x 2051) can then be captured
    in a CUDA graph, which allows no allocation, and the replay is bit-exact."""
    h, w = 2049, 2051
    a = oracle.gen("u8", 7300, (h, w))
    x = to_dev(a)
    y = torch.empty((h, w), dtype=torch.int32, device=cuda).view(torch.uint32)
    s = torch.cuda.Stream()
    L = _lib.load()
    with torch.cuda.stream(s):
        assert L.satgb_reserve(w, h, s.cuda_stream) == _lib.OK
        sat_gb300.sat(x, torch.uint32, out=y)  # descriptors encoded before the capture
        s.synchronize()
        y.zero_()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            sat_gb300.sat(x, torch.uint32, out=y)
        g.replay()
        s.synchronize()
    assert np.array_equal(to_np(y), oracle.sat_serial(a, np.uint32))


def test_batch_plan_float_and_reverse(cuda, oracle):
    rng = np.random.default_rng(6)
    ins, outs, arrs = [], [], []
    for i in range(20):
        h, w = int(rng.integers(1, 600)), int(rng.integers(1, 600))
        a = oracle.gen("f32u", 5000 + i, (h, w))
        arrs.append(a)
        ins.append(to_dev(a))
        outs.append(torch.empty((h, w), dtype=torch.float32, device="cuda"))
    for reverse in (False, True):
        plan = sat_gb300.BatchPlan(ins, outs, mode="compensated", reverse=reverse)
        plan.exec()
        plan.check()
        for a, o in zip(arrs, outs):
            _check_float(oracle, a, to_np(o), TOL_COMP, reverse=reverse)
        plan.close()


def test_autotune_records_and_results_stay_exact(cuda, oracle, tmp_path, monkeypatch):
    """satgb_autotune times every configuration on the caller's buffers, picks
    one, writes it to the tuning cache (one JSON object per line) and the
    next call with that size, which now uses it, is still bit-exact."""
    import json
    cache = tmp_path / "tune.jsonl"
    monkeypatch.setenv("SATGB_TUNE_CACHE", str(cache))
    a = oracle.gen("u8", 55, (700, 900))
    x = to_dev(a)
    y = torch.empty((700, 900), dtype=torch.int32, device=cuda).view(torch.uint32)
    best = sat_gb300.autotune(x, y)
    assert 0 <= best < len(sat_gb300.config_names())
    entries = [json.loads(line) for line in cache.read_text().splitlines()]
    mine = [e for e in entries if (e["in"], e["out"], e["wb"], e["hb"]) == (_lib.U8, _lib.U32, 10, 10)]
    assert mine and all(e["cfg"] == best for e in mine)
    out = to_np(sat_gb300.sat(x, torch.uint32))
    assert np.array_equal(bits(out), bits(oracle.sat_serial(a, np.uint32)))


def test_full_size_u8_properties_and_configs_agree(cuda):
    """8192 x 8192 u8 -> u32, the reference's largest case: the last row is
    the prefix of the column sums and the last column the prefix of the row
    sums (mod 2^32: the total of 2^26 bytes wraps), and the default tiles, the
    64-row two-CTA tiles and the 256-row direct-store tiles agree bit for bit."""
    g = torch.Generator(device=cuda).manual_seed(41)
    x = torch.randint(0, 256, (8192, 8192), dtype=torch.uint8, device=cuda, generator=g)
    s_def = sat_gb300.sat(x, torch.uint32)
    for cfg in (2, 4):
        sat_gb300.set_config(cfg)
        try:
            s2 = sat_gb300.sat(x, torch.uint32)
        finally:
            sat_gb300.set_config(-1)
        assert torch.equal(s_def.view(torch.int32), s2.view(torch.int32)), cfg
    col = x.to(torch.int64).sum(0).cumsum(0) & 0xFFFFFFFF
    row = x.to(torch.int64).sum(1).cumsum(0) & 0xFFFFFFFF
    assert torch.equal(s_def[-1].to(torch.int64), col)
    assert torch.equal(s_def[:, -1].to(torch.int64), row)


@pytest.mark.parametrize("cfg", [0, 1, 2, 3, 4, 5, 6])
def test_timeout_is_reported_and_context_survives(cuda, oracle, cfg):
    """A tile that never publishes makes its dependents hit the wait limit
    (every kernel: warp-specialized, pipelined, register-resident); the call
    reports SATGB_ERR_TIMEOUT and the next call is correct."""
    L = _lib.load()
    a = oracle.gen("u8", 77, (512, 512))
    x = to_dev(a)
    s = torch.cuda.Stream()
    try:
        sat_gb300.set_wait_limit_us(20_000)
        sat_gb300.set_config(cfg)
        assert L.satgb_debug_stall_tile(5) == 0
        with torch.cuda.stream(s):
            sat_gb300.scanrow_brlt(x, torch.uint32)
        L.satgb_debug_stall_tile(-1)
        # the next call, queued before anyone read the error, is unaffected
        with torch.cuda.stream(s):
            after = sat_gb300.scanrow_brlt(x, torch.uint32)
        with pytest.raises(sat_gb300.SatError) as ei:
            sat_gb300.stream_check(s)
        assert ei.value.status == _lib.ERR_TIMEOUT
        assert np.array_equal(to_np(after), oracle.sat_serial(a, np.uint32))
    finally:
        L.satgb_debug_stall_tile(-1)
        sat_gb300.set_wait_limit_us(2_000_000)
        sat_gb300.set_config(-1)
    with torch.cuda.stream(s):
        out = sat_gb300.scanrow_brlt(x, torch.uint32)
    sat_gb300.stream_check(s)  # the report was cleared by the check above
    assert np.array_equal(to_np(out), oracle.sat_serial(a, np.uint32))


def test_allocator_hook_failure(cuda, oracle):
    L = _lib.load()
    calls = []
    alloc = _lib._ALLOC_FN(lambda n, ctx: calls.append(n) or None)
    free = _lib._FREE_FN(lambda p, ctx: None)
    s = torch.cuda.Stream()  # fresh stream -> fresh workspace
    assert L.satgb_set_allocator(alloc, free, None) == 0
    try:
        x = to_dev(oracle.gen("u8", 1, (64, 64)))
        with torch.cuda.stream(s):
            with pytest.raises(sat_gb300.SatError) as ei:
                sat_gb300.scanrow_brlt(x, torch.uint32)
        assert ei.value.status == _lib.ERR_ALLOC
        assert calls
    finally:
        assert L.satgb_set_allocator(_lib._ALLOC_FN(), _lib._FREE_FN(), None) == 0


def test_launch_count_one_per_call(cuda, oracle):
    x = to_dev(oracle.gen("u8", 2, (1024, 1024)))
    before = sat_gb300.launch_count()
    for fn in ALGOS:
        fn(x, torch.uint32)
    assert sat_gb300.launch_count() - before == 3


@pytest.mark.slow
def test_full_size_8192_u8_u32_bit_exact(cuda, oracle):
    a = oracle.gen("u8", 8192, (8192, 8192))
    for fn in ALGOS:
        out = to_np(fn(to_dev(a), torch.uint32))
        assert np.array_equal(out, oracle.sat_serial(a, np.uint32)), fn.__name__


def _precision_8192(oracle, kind):
    a = oracle.gen(kind, 8193, (8192, 8192))
    x = to_dev(a)
    ref = oracle.sat_fp64(a)
    den = oracle.sat_fp64(a, absval=True)
    e_plain = oracle.err_stats(to_np(sat_gb300.sat(x, torch.float32)), ref, den)
    e_comp = oracle.err_stats(to_np(sat_gb300.sat(x, torch.float32, mode="compensated")), ref, den)
    print(f"\n[precision 8192^2 {kind}] plain {e_plain}  compensated {e_comp}")
    assert e_plain["max_rel_abs"] <= 1e-5, (kind, e_plain)
    return e_plain, e_comp


@pytest.mark.slow
def test_compensated_8192_uniform_within_1e6_relative(cuda, oracle):
    """U[0,1) inputs at 8192^2: every compensated SAT element is within 1e-6
    of the FP64 SAT relative to the element itself, |S - S64| / |S64|."""
    _, e_comp = _precision_8192(oracle, "f32u")
    assert e_comp["max_rel"] <= 1e-6, e_comp
    assert e_comp["max_rel_abs"] <= TOL_COMP, e_comp


@pytest.mark.slow
def test_compensated_8192_log_class_relative_to_sat_of_abs(cuda, oracle):
    """Magnitudes 10^U(-3,3) with random signs at 8192^2: sums cancel, so some
    exact elements are near 0 and no fixed-precision sum bounds the error
    relative to the element itself.  The stated bound for this class uses the
    condition-aware denominator SAT(|a|): |S - S64| / SAT(|a|)64 <= 2e-7
    (measured: about 3e-8); the relative error on elements is reported."""
    _, e_comp = _precision_8192(oracle, "f32log")
    assert e_comp["max_rel_abs"] <= TOL_COMP, e_comp


@pytest.mark.slow
def test_full_size_4096_f64(cuda, oracle):
    a = oracle.gen("f64u", 4096, (4096, 4096))
    out = to_np(sat_gb300.sat(to_dev(a), torch.float64))
    _check_float(oracle, a, out, TOL[np.dtype(np.float64)])


def test_cli_runs_reference_sizes(cuda):
    """`sat 0 1 0 4 2`: u8 -> u32 ScanRow-BRLT at 1024^2 and 2048^2, one CSV
    line per size in the reference's format."""
    import subprocess
    from sat_gb300 import build as B
    r = subprocess.run([B.cli_path(), "0", "1", "0", "4", "2", "--reps", "3"], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    assert lines[0].startswith("uchar-->uint, ScanRow-BRLT, LF_SCAN")
    for i, line in enumerate(lines[1:], start=1):
        w, h, rest = line.split(", ", 2)
        assert int(w) == int(h) == 1024 * i
        assert rest.startswith("total time = ")
        assert float(rest.split(", ")[-1]) > 0


SCAN_TORCH = {np.dtype(np.uint32): torch.uint32, np.dtype(np.int32): torch.int32,
              np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64}


@pytest.mark.parametrize("which", ["rows", "cols"])
def test_row_and_column_scans_all_pairs(cuda, oracle, which):
    """satgb_scan_rows / satgb_scan_cols (ScanX / ScanY as separate ops) against
    IntegralRow / IntegralStride: bit-exact for integer outputs; floats within
    1e-5 (f32) / 1e-13 (f64) of the FP64 scan, relative to the scan of |a|."""
    fn = sat_gb300.scan_rows if which == "rows" else sat_gb300.scan_cols
    ref = oracle.scan_rows if which == "rows" else oracle.scan_cols
    axis = 1 if which == "rows" else 0
    for name, (ti, to) in oracle.PAIRS.items():
        for i, shape in enumerate([(1, 1), (3, 700), (700, 3), (129, 257), (517, 769), (37, 1601)]):
            a = oracle.gen(PAIR_KINDS[ti], 3000 + i, shape)
            out = to_np(fn(to_dev(a), SCAN_TORCH[np.dtype(to)]))
            if np.dtype(to).kind in "iu":
                assert np.array_equal(bits(out), bits(ref(a, to))), (which, name, shape)
            else:
                exact = np.cumsum(a.astype(np.float64), axis=axis)
                den = np.cumsum(np.abs(a.astype(np.float64)), axis=axis)
                err = np.abs(out.astype(np.float64) - exact) / np.maximum(den, 1e-300)
                assert err.max() <= TOL[np.dtype(to)], (which, name, shape, err.max())


def test_scan_rows_transposed_all_pairs(cuda, oracle):
    """satgb_scan_rows_transposed (SerielScan::TestX: IntegralImageAllRow, then
    Transpose) against the oracle's row scan, transposed: bit-exact for integer
    outputs, floats within the scans' tolerance."""
    for name, (ti, to) in oracle.PAIRS.items():
        for i, shape in enumerate([(1, 1), (3, 700), (700, 3), (33, 129), (129, 257), (517, 769), (37, 1601)]):
            a = oracle.gen(PAIR_KINDS[ti], 3500 + i, shape)
            out = to_np(sat_gb300.scan_rows_transposed(to_dev(a), SCAN_TORCH[np.dtype(to)]))
            assert out.shape == (shape[1], shape[0])
            if np.dtype(to).kind in "iu":
                assert np.array_equal(bits(out), bits(oracle.scan_rows(a, to).T)), (name, shape)
            else:
                exact = np.cumsum(a.astype(np.float64), axis=1).T
                den = np.cumsum(np.abs(a.astype(np.float64)), axis=1).T
                err = np.abs(out.astype(np.float64) - exact) / np.maximum(den, 1e-300)
                assert err.max() <= TOL[np.dtype(to)], (name, shape, err.max())


def test_scan_rows_transposed_pitched_and_full_size(cuda, oracle):
    """Pitched input and output, odd pitches (no vector loads), and an
    8192 x 8192 u8 -> u32 check: the last output row is every input row's sum
    and the output equals the transposed row scan, mod 2^32."""
    a = oracle.gen("u8", 92, (333, 555))
    src = empty_pitched(333, 555, 641, torch.uint8)
    src.copy_(to_dev(a))
    dst = empty_pitched(555, 333, 400, torch.uint32, fill=-1)
    sat_gb300.scan_rows_transposed(src, torch.uint32, out=dst)
    assert np.array_equal(to_np(dst), oracle.scan_rows(a, np.uint32).T)
    # an output pitch of 401 elements: no 16-byte output vectors
    dst = empty_pitched(555, 333, 401, torch.uint32, fill=-1)
    sat_gb300.scan_rows_transposed(src, torch.uint32, out=dst)
    assert np.array_equal(to_np(dst), oracle.scan_rows(a, np.uint32).T)
    af = oracle.gen("f32n", 93, (333, 555))
    dstf = empty_pitched(555, 333, 333, torch.float64)
    sat_gb300.scan_rows_transposed(to_dev(af), torch.float64, out=dstf)
    exact = np.cumsum(af.astype(np.float64), axis=1).T
    assert np.abs(to_np(dstf) - exact).max() <= 1e-12 * np.abs(exact).max()
    g = torch.Generator(device=cuda).manual_seed(43)
    x = torch.randint(0, 256, (8192, 8192), dtype=torch.uint8, device=cuda, generator=g)
    t = sat_gb300.scan_rows_transposed(x, torch.uint32)
    r = sat_gb300.scan_rows(x, torch.uint32)
    assert torch.equal(t.view(torch.int32), r.view(torch.int32).t())
    rows = x.to(torch.int64).sum(1) & 0xFFFFFFFF
    assert torch.equal(t[-1].to(torch.int64), rows)


def test_golden_scans(cuda, golden_scans):
    """The CUDA row, transposed-row and column scans against the reference's
    own outputs (tests/golden/scans_golden.npz): bit-exact for integer outputs;
    floats within the scans' tolerance of the reference's sequential sums."""
    z, meta = golden_scans
    fns = (("__rows", sat_gb300.scan_rows, 1), ("__rows_t", sat_gb300.scan_rows_transposed, 1),
           ("__cols", sat_gb300.scan_cols, 0))
    for case in meta:
        a = z[case["key"] + "__in"]
        x = to_dev(a)
        for suffix, fn, axis in fns:
            ref = z[case["key"] + suffix]
            out = to_np(fn(x, SCAN_TORCH[ref.dtype]))
            if ref.dtype.kind in "iu":
                assert np.array_equal(bits(out), bits(ref)), (case["key"], suffix)
            else:
                den = np.cumsum(np.abs(a.astype(np.float64)), axis=axis)
                if suffix == "__rows_t":
                    den = den.T
                err = np.abs(out.astype(np.float64) - ref.astype(np.float64)) / np.maximum(den, 1e-300)
                assert err.max() <= TOL[ref.dtype], (case["key"], suffix, err.max())


def test_scans_pitched_and_full_size(cuda, oracle):
    """Pitched u8 -> u32 rows and columns, and an 8192 x 8192 check of
    sum(row scan) == sum(column scan) == the SAT's last element, mod 2^32."""
    a = oracle.gen("u8", 91, (333, 555))
    src = empty_pitched(333, 555, 640, torch.uint8)
    src.copy_(to_dev(a))
    for fn, ref in ((sat_gb300.scan_rows, oracle.scan_rows), (sat_gb300.scan_cols, oracle.scan_cols)):
        for opitch in (600, 601):  # 601: no 16-byte output vectors
            dst = empty_pitched(333, 555, opitch, torch.uint32, fill=-1)
            fn(src, torch.uint32, out=dst)
            assert np.array_equal(to_np(dst), ref(a, np.uint32))
    # in place (f32 -> f32 into its own buffer)
    af = oracle.gen("f32n", 94, (300, 1000))
    y = to_dev(af)
    sat_gb300.scan_rows(y, torch.float32, out=y)
    exact = np.cumsum(af.astype(np.float64), axis=1)
    den = np.cumsum(np.abs(af.astype(np.float64)), axis=1)
    assert (np.abs(to_np(y).astype(np.float64) - exact) / np.maximum(den, 1e-300)).max() <= TOL[np.dtype(np.float32)]
    x = torch.randint(0, 256, (8192, 8192), dtype=torch.uint8, device=cuda)
    r = sat_gb300.scan_rows(x, torch.uint32)
    c = sat_gb300.scan_cols(x, torch.uint32)
    s = sat_gb300.sat(x, torch.uint32)
    total = int(x.to(torch.int64).sum().item()) % (1 << 32)
    assert int(r[:, -1].view(torch.int32).to(torch.int64).remainder(1 << 32).sum().item()) % (1 << 32) == total
    assert int(c[-1, :].view(torch.int32).to(torch.int64).remainder(1 << 32).sum().item()) % (1 << 32) == total
    assert int(s[-1, -1].view(torch.int32).to(torch.int64).item()) % (1 << 32) == total


@pytest.mark.slow
@pytest.mark.parametrize("pitched", [True, False])
def test_batch512_bit_exact(cuda, oracle, pitched):
    """The batch workload exactly as the bench builds it: 512 u8 images with
    widths and heights log-uniform in [64, 4096] (about 590 M pixels), rows
    pitched to 128 bytes or packed, one graph replay of the plan with its
    untuned configurations and one after the batch autotuner picked a
    configuration per size class; every image bit-exact against the oracle."""
    from bench import build_batch
    xs, ys, _ = build_batch(cuda, pitched=pitched)
    plan = sat_gb300.BatchPlan(xs, ys)
    cls = plan.classes()
    assert cls[0]["images"] > 0 and cls[1]["images"] > 0 and cls[0]["images"] + cls[1]["images"] == 512
    for rep, tuned in ((0, False), (1, True)):
        if tuned:
            chosen = plan.autotune()  # every configuration of each class, timed on these images
            assert [c["config"] for c in plan.classes()] == list(chosen)
        for y in ys:
            y.view(torch.int32).fill_(-1)
        plan.exec()
        plan.check()
        for i, (x, y) in enumerate(zip(xs, ys)):
            a = to_np(x)
            assert np.array_equal(bits(to_np(y)), bits(oracle.sat_serial(a, np.uint32))), (tuned, i)
    plan.close()


@pytest.mark.slow
def test_stress_32768_u8_u32_bit_exact(cuda, oracle):
    """32768 x 32768 u8 -> u32 (2^30 pixels; sums wrap mod 2^32 many times)
    bit-exact against the oracle."""
    a = oracle.gen("u8", 32768, (32768, 32768))
    x = to_dev(a)
    out = sat_gb300.sat(x, torch.uint32)
    del x
    got = to_np(out)
    del out
    assert np.array_equal(got, oracle.sat_serial(a, np.uint32))


@pytest.mark.slow
def test_stress_16384_compensated_f32(cuda, oracle):
    """16384 x 16384 U[0,1) through the compensated f32 SAT: within 1e-6 of
    the FP64 SAT relative to each element, and 2e-7 relative to SAT(|a|)."""
    a = oracle.gen("f32u", 16384, (16384, 16384))
    comp = to_np(sat_gb300.sat(to_dev(a), torch.float32, mode="compensated"))
    e = oracle.err_stats(comp, oracle.sat_fp64(a), oracle.sat_fp64(a, absval=True))
    print(f"\n[precision 16384^2 f32u compensated] {e}")
    assert e["max_rel"] <= 1e-6, e
    assert e["max_rel_abs"] <= TOL_COMP, e
