"""Generates tests/golden/sat_golden.npz from the reference's OWN CPU integral
image (pengdada/SAT integralImage/integralImage.h:105-124, IntegralImageSerial),
compiled from the reference checkout by ``make -C oracle ref`` into
oracle/_ref/libref_sat.so.

The reference ships no golden vectors or known-answer files (its Compare()
returns true before comparing, integralImage.h:268), so these fixtures are the
reference run on seeded inputs.  They pin the C restatement in
oracle/sat_oracle.c (tests/test_oracle.py) and the CUDA path
(tests/test_gpu_parity.py) on machines where the reference is absent.

Small cases store input and output arrays; the 1024x1024 cases (the
reference's own smallest benchmark size, ScanRow-BRLT.cu:272-273) store the
generator spec plus SHA-256 digests of input and output.

Run from the repository root, with SATGB_REF_DIR naming the reference checkout's
integralImage/ directory:  SATGB_REF_DIR=<checkout>/integralImage python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "sat_golden.npz")

KIND = {np.uint8: "u8", np.int8: "i8", np.int32: "i32", np.uint32: "u32",
        np.float32: "f32u", np.float64: "f64u"}
SMALL_SIZES = [(1, 1), (1, 13), (13, 1), (31, 33), (67, 129)]
BIG = [
    # (name, pair, gen kind, seed, (h, w))
    ("u8_u32_1024_uniform", "u8_u32", "u8", 1, (1024, 1024)),
    ("u8_u32_1024_binary", "u8_u32", "bin", 2, (1024, 1024)),
    ("u8_u32_997x1000", "u8_u32", "u8", 3, (997, 1000)),
    ("u8_f32_1024_uniform", "u8_f32", "u8", 4, (1024, 1024)),
    ("f32_f32_1024_uniform", "f32_f32", "f32u", 5, (1024, 1024)),
    ("f64_f64_1024_uniform", "f64_f64", "f64u", 6, (1024, 1024)),
    ("u32_u32_1024_wrap", "u32_u32", "u32", 7, (1024, 1024)),
]


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main() -> None:
    O.build(with_ref=True)
    if O.ref_lib() is None:
        raise SystemExit("the reference's CPU code is not built (oracle/_ref/libref_sat.so)")
    arrays = {}
    meta = {"small": [], "big": []}
    seed = 100
    for name, (ti, to) in O.PAIRS.items():
        kinds = [KIND[ti]]
        if ti is np.float32:
            kinds.append("f32log")
        for kind in kinds:
            for (h, w) in SMALL_SIZES:
                seed += 1
                a = O.gen(kind, seed, (h, w))
                r = O.ref_serial(a, to)
                key = f"{name}_{kind}_{h}x{w}"
                arrays[key + "__in"] = a
                arrays[key + "__out"] = r
                meta["small"].append({"key": key, "pair": name, "kind": kind, "seed": seed, "h": h, "w": w})
    for (key, pair, kind, sd, (h, w)) in BIG:
        ti, to = O.PAIRS[pair]
        a = O.gen(kind, sd, (h, w)).astype(ti)
        r = O.ref_serial(a, to)
        meta["big"].append({"key": key, "pair": pair, "kind": kind, "seed": sd, "h": h, "w": w,
                            "in_sha256": sha(a), "out_sha256": sha(r),
                            "out_last": r[-1, -1].item(), "out_row0_last": r[0, -1].item()})
    arrays["__meta__"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {OUT}: {len(meta['small'])} small cases, {len(meta['big'])} digest cases")


if __name__ == "__main__":
    main()
