"""Generate tests/golden/golden.json from the reference library itself.

The reference (Natural_Number) has no tests or golden vectors of its own, so
the fixtures are produced by running the reference, compiled from its own
sources by oracle/build_ref.sh (x86-64, reference present), on seeded inputs
(natural_number_gb300.synth.limbs).  Each result is stored as its limb count
plus the SHA-256 of its little-endian limb bytes (decimal strings: length plus
SHA-256 of the ASCII digits), so the file stays small while pinning every bit.

    python tests/golden/make_golden.py          # standard fixture set (~1 min)
    python tests/golden/make_golden.py --big    # also 2^27-limb mul/sqr and pi/e at 1e8 digits
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from natural_number_gb300.synth import limbs  # noqa: E402
from oracle import Oracle, build_reference  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")


def digest(x: np.ndarray) -> dict:
    x = np.ascontiguousarray(x, dtype="<u8")
    return {"n": int(x.size), "sha256": hashlib.sha256(x.tobytes()).hexdigest()}


def sdigest(s: str) -> dict:
    return {"len": len(s), "sha256": hashlib.sha256(s.encode()).hexdigest(), "head": s[:32]}


MUL_CASES = [(1, 1), (2, 1), (5, 3), (31, 17), (32, 32), (47, 33), (100, 50), (383, 383), (383, 384),
             (384, 384), (385, 1000), (1000, 385), (2048, 2048), (4096, 4096), (5000, 300), (20000, 13000),
             (65536, 65536), (100000, 3), (1 << 17, 1 << 17), (70001, 65536)]
SQR_CASES = [1, 2, 31, 32, 47, 48, 49, 100, 383, 384, 385, 1000, 4096, 30000, 1 << 17]
# (na, nb, scale, size); size-1 > 2^scale selects the reference's wrap mode.
RAW_CASES = [(600, 600, 10, 1200), (700, 500, 10, 1200), (1000, 1000, 10, 2000), (1000, 1000, 11, 2000),
             (1024, 1024, 10, 2048), (1024, 1024, 11, 2049), (2000, 1500, 11, 3500), (3000, 2000, 12, 5000),
             (4096, 100, 12, 4196), (4096, 4096, 12, 8192), (4096, 4096, 13, 8192), (1 << 15, 1 << 15, 15, 1 << 16),
             (1 << 15, 9000, 15, (1 << 15) + 9000), (20000, 20000, 16, 40000)]
DIV_CASES = [(2, 1), (3, 2), (10, 3), (100, 99), (1000, 2), (1000, 999), (2000, 1000), (5000, 1200),
             (20000, 10000), (70000, 30000), (3000, 2999), (40000, 17), (1 << 16, 1 << 15), (300000, 100000)]
RECIP_CASES = [(3, 6), (10, 30), (100, 201), (1000, 2001), (5000, 9000), (30000, 60001)]
DEC_CASES = [1, 2, 100, 3000, 20000]
PI_CASES = [(1 << 7, 60, 1000), (1 << 10, 600, 10000), (1 << 13, 6000, 100000), (1 << 17, 60000, 1000000),
            (1 << 20, 600000, 10000000)]
E_CASES = [(1 << 9, 1000), (1 << 12, 10000), (1 << 15, 100000), (1 << 18, 1000000), (1 << 21, 10000000)]
BIG_MUL = [(1 << 24, 1 << 24), (1 << 27, 1 << 27)]
BIG_SQR = [1 << 24, 1 << 27]
BIG_PI = [(1 << 23, 6000000, 100000000)]
BIG_E = [(1 << 24, 100000000)]


def seed_a(n: int, k: int = 1) -> int:
    return 1000 * k + n


def seed_b(n: int, k: int = 1) -> int:
    return 7777 * k + n


def generate(big: bool) -> dict:
    R = Oracle("ref")
    g: dict = {"generator": "reference compiled from its sources (oracle/build_ref.sh)",
               "inputs": "natural_number_gb300.synth.limbs(seed, n)",
               "mul": [], "sqr": [], "ntt_raw": [], "ntt_forward": [], "root_tables": [],
               "div": [], "div_edge": [], "reciprocal2": [], "reciprocal3": [], "pow": [],
               "to_dec": [], "pi": [], "e": []}
    for na, nb in MUL_CASES:
        for k in (1, 2):
            a, b = limbs(seed_a(na, k), na), limbs(seed_b(nb, k), nb)
            g["mul"].append({"na": na, "nb": nb, "seed_a": seed_a(na, k), "seed_b": seed_b(nb, k),
                             "out": digest(R.mul(a, b))})
    for n in SQR_CASES:
        a = limbs(seed_a(n), n)
        g["sqr"].append({"n": n, "seed": seed_a(n), "out": digest(R.sqr(a))})
    for na, nb, s, size in RAW_CASES:
        a, b = limbs(seed_a(na), na), limbs(seed_b(nb), nb)
        g["ntt_raw"].append({"na": na, "nb": nb, "seed_a": seed_a(na), "seed_b": seed_b(nb), "scale": s,
                             "size": size, "out": digest(R.ntt_mul_raw(a, b, s, size))})
    P = [27 << 56 | 1, 58 << 56 | 1, 87 << 56 | 1]
    for s, n in ((10, 500), (12, 2048), (14, 5000), (14, 16384)):
        a = limbs(seed_a(n), n)
        f = R.ntt_forward(a, s)
        canon = np.stack([f[i] % np.uint64(P[i]) for i in range(3)])
        g["ntt_forward"].append({"scale": s, "n": n, "seed": seed_a(n), "raw": digest(f.ravel()),
                                 "canonical": digest(canon.ravel())})
    for s in (12, 16):
        for prime in range(3):
            for inv in (0, 1):
                g["root_tables"].append({"scale": s, "prime": prime, "inverse": inv,
                                         "out": digest(R.root_table(s, prime, bool(inv)))})
    for na, nb in DIV_CASES:
        for k in (1, 2):
            a, b = limbs(seed_a(na, k), na), limbs(seed_b(nb, k), nb)
            q, r = R.div(a, b)
            g["div"].append({"na": na, "nb": nb, "seed_a": seed_a(na, k), "seed_b": seed_b(nb, k),
                             "q": digest(q), "r": digest(r)})
    edge = {"zero_by_zero": ([0], [0]), "x_by_zero": ([5, 7], [0]), "zero_by_x": ([0], [3, 1]),
            "small_by_big": ([9, 9], [1, 1, 1]), "equal": ([4, 5, 6], [4, 5, 6]),
            "one_limb": (list(limbs(5, 50)), [12345]), "pow2_divisor": (list(limbs(6, 40)), [0, 0, 1]),
            "top_bit_divisor": (list(limbs(7, 60)), [1, 2**63]),
            "max_limbs": ([2**64 - 1] * 70, [2**64 - 1] * 33)}
    for name, (a, b) in edge.items():
        q, r = R.div(np.array(a, dtype=np.uint64), np.array(b, dtype=np.uint64))
        g["div_edge"].append({"name": name, "a": [str(x) for x in a], "b": [str(x) for x in b],
                              "q": digest(q), "r": digest(r)})
    for n, dsz in RECIP_CASES:
        d = limbs(seed_a(n), n).copy()
        d[-1] = 1  # the reciprocals require a top limb of exactly 1 (natural.h:575, 619)
        g["reciprocal2"].append({"n": n, "seed": seed_a(n), "divd_size": dsz, "out": digest(R.reciprocal2(d, dsz))})
        g["reciprocal3"].append({"n": n, "seed": seed_a(n), "divd_size": dsz, "out": digest(R.reciprocal3(d, dsz))})
    for base, e in ((2, 65536), (3, 1000), (10, 10000), (12345678901, 777)):
        p = R.pow(np.array([base], dtype=np.uint64), e)
        g["pow"].append({"base": base, "e": e, "out": digest(p), "dec": sdigest(R.to_dec(p))})
    for n in DEC_CASES:
        g["to_dec"].append({"n": n, "seed": seed_a(n), "out": sdigest(R.to_dec(limbs(seed_a(n), n)))})
    for terms, acc, digits in PI_CASES:
        t = time.time()
        g["pi"].append({"terms": terms, "acc": acc, "digits": digits, "out": sdigest(R.pi_dec(terms, acc, digits)),
                        "ref_seconds": round(time.time() - t, 3)})
    for terms, digits in E_CASES:
        t = time.time()
        g["e"].append({"terms": terms, "digits": digits, "out": sdigest(R.e_dec(terms, digits)),
                       "ref_seconds": round(time.time() - t, 3)})
    if big:
        g["big_mul"], g["big_sqr"], g["big_pi"], g["big_e"] = [], [], [], []
        for na, nb in BIG_MUL:
            a, b = limbs(seed_a(na), na), limbs(seed_b(nb), nb)
            t = time.time()
            out = digest(R.mul(a, b))
            g["big_mul"].append({"na": na, "nb": nb, "seed_a": seed_a(na), "seed_b": seed_b(nb), "out": out,
                                 "ref_seconds": round(time.time() - t, 3)})
        for n in BIG_SQR:
            a = limbs(seed_a(n), n)
            t = time.time()
            g["big_sqr"].append({"n": n, "seed": seed_a(n), "out": digest(R.sqr(a)),
                                 "ref_seconds": round(time.time() - t, 3)})
        for terms, acc, digits in BIG_PI:
            t = time.time()
            g["big_pi"].append({"terms": terms, "acc": acc, "digits": digits,
                                "out": sdigest(R.pi_dec(terms, acc, digits)), "ref_seconds": round(time.time() - t, 3)})
        for terms, digits in BIG_E:
            t = time.time()
            g["big_e"].append({"terms": terms, "digits": digits, "out": sdigest(R.e_dec(terms, digits)),
                               "ref_seconds": round(time.time() - t, 3)})
    return g


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--big", action="store_true")
    args = ap.parse_args()
    if build_reference() is None:
        sys.exit("reference not buildable on this host")
    g = generate(args.big)
    if not args.big and os.path.exists(OUT):
        old = json.load(open(OUT))
        for k in ("big_mul", "big_sqr", "big_pi", "big_e"):
            if k in old:
                g[k] = old[k]
    with open(OUT, "w") as f:
        json.dump(g, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
