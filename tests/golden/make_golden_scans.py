"""Generates tests/golden/scans_golden.npz from the reference's OWN CPU row and
column scans (pengdada/SAT integralImage/integralImage.h): IntegralImageAllRow
(:148-160, IntegralRow on every row), IntegralImageAllRow followed by Transpose
(:280-288; what SerielScan::TestX compares its transposed row scan with,
BRLT-Scan.cu:176-180) and IntegralStride down every column (:91-101), all
compiled from the reference checkout by ``make -C oracle ref`` into
oracle/_ref/libref_sat.so.

The fixtures pin the oracle's scans (tests/test_oracle.py) and the CUDA scans
(tests/test_gpu_parity.py) on machines where the reference is absent.

Run from the repository root, with SATGB_REF_DIR naming the reference checkout's
integralImage/ directory:  SATGB_REF_DIR=<checkout>/integralImage python tests/golden/make_golden_scans.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "scans_golden.npz")

KIND = {np.uint8: "u8", np.int8: "i8", np.int32: "i32", np.uint32: "u32",
        np.float32: "f32u", np.float64: "f64u"}
SIZES = [(1, 1), (1, 13), (13, 1), (31, 33), (40, 70)]


def main() -> None:
    O.build(with_ref=True)
    if O.ref_lib() is None:
        raise SystemExit("the reference's CPU code is not built (oracle/_ref/libref_sat.so)")
    arrays = {}
    meta = []
    seed = 500
    for name, (ti, to) in O.PAIRS.items():
        for (h, w) in SIZES:
            seed += 1
            a = O.gen(KIND[ti], seed, (h, w))
            key = f"{name}_{h}x{w}"
            arrays[key + "__in"] = a
            arrays[key + "__rows"] = O.ref_scan_rows(a, to)
            arrays[key + "__rows_t"] = O.ref_scan_rows_transposed(a, to)
            arrays[key + "__cols"] = O.ref_scan_cols(a, to)
            meta.append({"key": key, "pair": name, "seed": seed, "h": h, "w": w})
    arrays["__meta__"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {OUT}: {len(meta)} cases")


if __name__ == "__main__":
    main()
