"""The oracle (CPU restatement of the reference's integral image) is pinned
against the reference itself: the committed golden vectors (made by running
the reference's own IntegralImageSerial) and, where the reference checkout is
present, the reference compiled live into oracle/_ref/."""
import hashlib

import numpy as np
import pytest


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint8)


def test_golden_small_cases_bit_exact(oracle, golden):
    z, meta = golden
    assert len(meta["small"]) >= 60
    for case in meta["small"]:
        a = z[case["key"] + "__in"]
        r = z[case["key"] + "__out"]
        out_dtype = oracle.PAIRS[case["pair"]][1]
        s = oracle.sat_serial(a, out_dtype)
        assert s.dtype == r.dtype
        assert np.array_equal(_bits(s), _bits(r)), case["key"]
        # the OpenMP restatement of IntegralImageParallel gives the same bits
        p = oracle.sat_parallel(a, out_dtype, nthreads=3)
        assert np.array_equal(_bits(p), _bits(r)), case["key"]


def test_golden_inputs_regenerate(oracle, golden):
    """The seeded generator reproduces the committed inputs bit for bit."""
    z, meta = golden
    for case in meta["small"]:
        if case["kind"] == "f32log":
            continue  # uses libm pow; its input is stored, not regenerated
        a = oracle.gen(case["kind"], case["seed"], (case["h"], case["w"]))
        assert np.array_equal(_bits(a), _bits(z[case["key"] + "__in"])), case["key"]


def test_golden_digest_cases(oracle, golden):
    _, meta = golden
    for case in meta["big"]:
        ti, to = oracle.PAIRS[case["pair"]]
        a = oracle.gen(case["kind"], case["seed"], (case["h"], case["w"])).astype(ti)
        assert hashlib.sha256(a.tobytes()).hexdigest() == case["in_sha256"], case["key"]
        s = oracle.sat_serial(a, to)
        assert hashlib.sha256(s.tobytes()).hexdigest() == case["out_sha256"], case["key"]


def test_numpy_restatement_matches_c(oracle):
    for name, (ti, to) in oracle.PAIRS.items():
        kind = {np.uint8: "u8", np.int8: "i8", np.int32: "i32", np.uint32: "u32",
                np.float32: "f32u", np.float64: "f64u"}[ti]
        a = oracle.gen(kind, 11, (9, 23), use_c=False)
        assert np.array_equal(_bits(oracle.sat_serial_np(a, to)), _bits(oracle.sat_serial(a, to))), name


def test_generator_c_equals_numpy(oracle):
    for kind in ("u8", "u32", "f32u", "f64u"):
        a = oracle.gen(kind, 5, (17, 61))
        b = oracle.gen(kind, 5, (17, 61), use_c=False)
        assert np.array_equal(_bits(a), _bits(b)), kind


def test_u32_wraps_mod_2_32(oracle):
    a = np.full((4, 4), 0xFFFFFFFF, dtype=np.uint32)
    s = oracle.sat_serial(a, np.uint32)
    exact = (np.arange(1, 5)[:, None] * np.arange(1, 5)[None, :]) * 0xFFFFFFFF
    assert np.array_equal(s.astype(np.uint64), (exact % (1 << 32)).astype(np.uint64))


def test_empty_and_degenerate(oracle):
    a = np.zeros((0, 5), dtype=np.uint8)
    assert oracle.sat_serial(a, np.uint32).shape == (0, 5)
    a = np.array([[7]], dtype=np.uint8)
    assert oracle.sat_serial(a, np.uint32)[0, 0] == 7


def test_pitched_input(oracle):
    base = oracle.gen("u8", 3, (20, 40))
    view = base[:, 3:31]  # pitch 40, width 28
    ref = oracle.sat_serial(np.ascontiguousarray(view), np.uint32)
    assert np.array_equal(oracle.sat_serial(view, np.uint32), ref)


def test_fp64_oracle_exact_on_integers(oracle):
    a = oracle.gen("u8", 9, (300, 200))
    d = oracle.sat_fp64(a)
    s = a.astype(np.int64).cumsum(0).cumsum(1)
    assert np.array_equal(d, s.astype(np.float64))


def test_fp64_oracle_reverse_is_flipped_forward(oracle):
    a = oracle.gen("f32log", 4, (50, 70))
    r = oracle.sat_fp64(a, reverse=True)
    f = oracle.sat_fp64(np.ascontiguousarray(a[::-1, ::-1]))[::-1, ::-1]
    assert np.array_equal(r, f)
    ri = oracle.sat_reverse(oracle.gen("u8", 4, (50, 70)), np.uint32)
    fi = oracle.sat_serial(np.ascontiguousarray(oracle.gen("u8", 4, (50, 70))[::-1, ::-1]), np.uint32)[::-1, ::-1]
    assert np.array_equal(ri, fi)


def test_fp64_oracle_close_to_longdouble(oracle):
    a = oracle.gen("f32log", 12, (40, 40))
    d = oracle.sat_fp64(a)
    ld = a.astype(np.longdouble).cumsum(0).cumsum(1)
    scale = oracle.sat_fp64(a, absval=True)
    assert np.max(np.abs(d - ld.astype(np.float64)) / scale) < 1e-15


def test_err_stats(oracle):
    a = oracle.gen("f32u", 2, (64, 64))
    d = oracle.sat_fp64(a)
    st = oracle.err_stats(d.astype(np.float32), d, oracle.sat_fp64(a, absval=True))
    assert st["max_rel"] < 6e-8 and st["max_rel_abs"] < 6e-8


def test_reference_live_matches_port(oracle):
    """Where the reference checkout is present its own CPU code is compiled
    into oracle/_ref/ and must agree with the restatement bit for bit."""
    if oracle.ref_lib() is None:
        pytest.skip("reference CPU code not built here (no reference checkout)")
    kinds = {np.uint8: "u8", np.int8: "i8", np.int32: "i32", np.uint32: "u32",
             np.float32: "f32u", np.float64: "f64u"}
    for name, (ti, to) in oracle.PAIRS.items():
        for shape in [(1, 1), (5, 300), (300, 5), (129, 131)]:
            a = oracle.gen(kinds[ti], 21, shape)
            assert np.array_equal(_bits(oracle.ref_serial(a, to)), _bits(oracle.sat_serial(a, to))), (name, shape)
    for t, kind in [(np.uint32, "u32"), (np.int32, "i32"), (np.float32, "f32u"), (np.float64, "f64u")]:
        a = oracle.gen(kind, 22, (77, 91))
        assert np.array_equal(_bits(oracle.ref_parallel(a)), _bits(oracle.sat_parallel(a, t)))


def test_oracle_row_and_column_scans(oracle):
    """IntegralRow / IntegralStride restated (integralImage.h:74-101): integer
    pairs equal numpy's cumsum in the output type (wrapping mod 2^32)."""
    for name in ("u8_u32", "i8_i32", "i32_i32", "u32_u32"):
        ti, to = oracle.PAIRS[name]
        kind = {np.uint8: "u8", np.int8: "i8", np.int32: "i32", np.uint32: "u32"}[ti]
        a = oracle.gen(kind, 77, (41, 67)).astype(ti)
        acc = a.astype(np.int64).astype(np.uint32)
        with np.errstate(over="ignore"):
            assert np.array_equal(oracle.scan_rows(a, to).view(np.uint32), np.cumsum(acc, axis=1, dtype=np.uint32))
            assert np.array_equal(oracle.scan_cols(a, to).view(np.uint32), np.cumsum(acc, axis=0, dtype=np.uint32))


def test_reference_live_scans_match_port(oracle):
    """The row scan, the transposed row scan and the column scan of the
    restatement against the reference's own IntegralImageAllRow,
    AllRow + Transpose (SerielScan::TestX's check) and IntegralStride, bit for
    bit, every pair (floats included: the same order of additions)."""
    if oracle.ref_lib() is None:
        pytest.skip("reference CPU code not built here (no reference checkout)")
    kinds = {np.uint8: "u8", np.int8: "i8", np.int32: "i32", np.uint32: "u32",
             np.float32: "f32u", np.float64: "f64u"}
    for name, (ti, to) in oracle.PAIRS.items():
        for shape in [(1, 1), (5, 300), (300, 5), (129, 131)]:
            a = oracle.gen(kinds[ti], 23, shape)
            rows = oracle.scan_rows(a, to)
            assert np.array_equal(_bits(oracle.ref_scan_rows(a, to)), _bits(rows)), (name, shape)
            assert np.array_equal(_bits(oracle.ref_scan_rows_transposed(a, to)),
                                  _bits(np.ascontiguousarray(rows.T))), (name, shape)
            assert np.array_equal(_bits(oracle.ref_scan_cols(a, to)), _bits(oracle.scan_cols(a, to))), (name, shape)


def test_golden_scans_bit_exact(oracle, golden_scans):
    """The restatement's row, transposed-row and column scans against the
    reference's own outputs (tests/golden/scans_golden.npz), every pair, bit
    for bit."""
    z, meta = golden_scans
    for case in meta:
        a = z[case["key"] + "__in"]
        to = z[case["key"] + "__rows"].dtype
        rows = oracle.scan_rows(a, to)
        assert np.array_equal(_bits(rows), _bits(z[case["key"] + "__rows"])), case["key"]
        assert np.array_equal(_bits(np.ascontiguousarray(rows.T)), _bits(z[case["key"] + "__rows_t"])), case["key"]
        assert np.array_equal(_bits(oracle.scan_cols(a, to)), _bits(z[case["key"] + "__cols"])), case["key"]
