"""The oracle (CPU restatement) against the reference's own outputs.

tests/golden/golden.json was produced by running the reference library itself
(tests/golden/make_golden.py); these tests pin the oracle to it bit for bit,
so the GPU parity tests can trust the oracle on inputs the fixtures do not hold.
"""
import hashlib

import numpy as np
import pytest

from natural_number_gb300.synth import limbs

P = [27 << 56 | 1, 58 << 56 | 1, 87 << 56 | 1]


def digest(x):
    x = np.ascontiguousarray(x, dtype="<u8")
    return {"n": int(x.size), "sha256": hashlib.sha256(x.tobytes()).hexdigest()}


def sdig(s):
    return {"len": len(s), "sha256": hashlib.sha256(s.encode()).hexdigest(), "head": s[:32]}


def test_mul(golden, oracle):
    for c in golden["mul"]:
        a, b = limbs(c["seed_a"], c["na"]), limbs(c["seed_b"], c["nb"])
        assert digest(oracle.mul(a, b)) == c["out"], (c["na"], c["nb"])


def test_sqr(golden, oracle):
    for c in golden["sqr"]:
        assert digest(oracle.sqr(limbs(c["seed"], c["n"]))) == c["out"], c["n"]


def test_ntt_raw_including_wrap(golden, oracle):
    wraps = 0
    for c in golden["ntt_raw"]:
        a, b = limbs(c["seed_a"], c["na"]), limbs(c["seed_b"], c["nb"])
        out = oracle.ntt_mul_raw(a, b, c["scale"], c["size"])
        assert digest(out) == c["out"], c
        wraps += c["size"] - 1 > (1 << c["scale"])
    assert wraps >= 3


def test_ntt_forward_residues(golden, oracle):
    for c in golden["ntt_forward"]:
        f = oracle.ntt_forward(limbs(c["seed"], c["n"]), c["scale"])
        assert digest(f.ravel()) == c["raw"]
        canon = np.stack([f[i] % np.uint64(P[i]) for i in range(3)])
        assert digest(canon.ravel()) == c["canonical"]


def test_root_tables(golden, oracle):
    for c in golden["root_tables"]:
        t = oracle.root_table(c["scale"], c["prime"], bool(c["inverse"]))
        assert digest(t) == c["out"], c


def test_div(golden, oracle):
    for c in golden["div"]:
        a, b = limbs(c["seed_a"], c["na"]), limbs(c["seed_b"], c["nb"])
        q, r = oracle.div(a, b)
        assert digest(q) == c["q"] and digest(r) == c["r"], (c["na"], c["nb"])


def test_div_edge_cases(golden, oracle):
    names = set()
    for c in golden["div_edge"]:
        a = np.array([int(x) for x in c["a"]], dtype=np.uint64)
        b = np.array([int(x) for x in c["b"]], dtype=np.uint64)
        q, r = oracle.div(a, b)
        assert digest(q) == c["q"] and digest(r) == c["r"], c["name"]
        names.add(c["name"])
    assert {"zero_by_zero", "x_by_zero", "small_by_big"} <= names


def test_reciprocals(golden, oracle):
    for kind in ("reciprocal2", "reciprocal3"):
        for c in golden[kind]:
            d = limbs(c["seed"], c["n"]).copy()
            d[-1] = 1
            out = getattr(oracle, kind)(d, c["divd_size"])
            assert digest(out) == c["out"], (kind, c)


def test_pow_and_decimal(golden, oracle):
    for c in golden["pow"]:
        p = oracle.pow(np.array([c["base"]], dtype=np.uint64), c["e"])
        assert digest(p) == c["out"]
        assert sdig(oracle.to_dec(p)) == c["dec"]
    for c in golden["to_dec"]:
        assert sdig(oracle.to_dec(limbs(c["seed"], c["n"]))) == c["out"]


@pytest.mark.parametrize("idx", range(5))
def test_pi_digits(golden, oracle, idx):
    c = golden["pi"][idx]
    assert sdig(oracle.pi_dec(c["terms"], c["acc"], c["digits"])) == c["out"]


@pytest.mark.parametrize("idx", range(5))
def test_e_digits(golden, oracle, idx):
    c = golden["e"][idx]
    assert sdig(oracle.e_dec(c["terms"], c["digits"])) == c["out"]


def test_oracle_against_python_int(oracle):
    """Independent exact check of products and quotients with Python integers."""
    from oracle import to_int
    for na, nb, seed in ((7, 5, 1), (400, 390, 2), (3000, 1700, 3)):
        a, b = limbs(seed, na), limbs(seed + 100, nb)
        A, B = to_int(a), to_int(b)
        assert to_int(oracle.mul(a, b)) == A * B
        q, r = oracle.div(a, b)
        assert to_int(q) == A // B and to_int(r) == A % B


# Divisions on which the reference's own Newton division breaks its size
# preconditions and aborts (natural.h:670-676): (seed_a, n_a, seed_b, n_b).
REFERENCE_ABORTS = [(5046, 7406, 5047, 3703), (19141, 4406, 19142, 2203)]


def test_divisions_the_reference_cannot_do_are_exact(oracle):
    """The oracle detects the broken precondition and finishes with an exact
    long division; the results are checked against Python integers."""
    from oracle import to_int
    for sa, na, sb, nb in REFERENCE_ABORTS:
        a, b = limbs(sa, na), limbs(sb, nb)
        q, r = oracle.div(a, b)
        A, B = to_int(a), to_int(b)
        assert to_int(q) == A // B and to_int(r) == A % B
