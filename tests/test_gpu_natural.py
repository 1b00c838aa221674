"""GPU parity of the natural-level algorithms (division with the Newton
reciprocal, reciprocals, power, decimal output, pi and e) against the
reference's own outputs and the oracle.  Every product runs on the GPU."""
import hashlib
import os
import subprocess

import numpy as np
import pytest

from gpu_util import digest
from natural_number_gb300.synth import limbs

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def sdig(s):
    return {"len": len(s), "sha256": hashlib.sha256(s.encode()).hexdigest(), "head": s[:32]}


@pytest.fixture(scope="module")
def ctx():
    import natural_number_gb300 as nn
    c = nn.Context(0)
    yield c
    c.close()


def test_div_golden(ctx, golden):
    for c in golden["div"]:
        a, b = limbs(c["seed_a"], c["na"]), limbs(c["seed_b"], c["nb"])
        q, r = ctx.div(a, b)
        assert digest(q) == c["q"] and digest(r) == c["r"], (c["na"], c["nb"])


def test_div_edge_cases_golden(ctx, golden):
    for c in golden["div_edge"]:
        a = np.array([int(x) for x in c["a"]], dtype=np.uint64)
        b = np.array([int(x) for x in c["b"]], dtype=np.uint64)
        q, r = ctx.div(a, b)
        assert digest(q) == c["q"] and digest(r) == c["r"], c["name"]


@pytest.mark.parametrize("na,nb", [(600, 599), (3000, 1000), (20001, 9000), (1 << 17, 1 << 16), (100000, 384)])
def test_div_vs_oracle(ctx, oracle, na, nb):
    a, b = limbs(na + 5, na), limbs(nb + 9, nb)
    q1, r1 = ctx.div(a, b)
    q2, r2 = oracle.div(a, b)
    assert np.array_equal(q1, q2) and np.array_equal(r1, r2)


def test_reciprocals_golden(ctx, golden):
    for kind, variant in (("reciprocal2", 2), ("reciprocal3", 3)):
        for c in golden[kind]:
            d = limbs(c["seed"], c["n"]).copy()
            d[-1] = 1
            assert digest(ctx.reciprocal(d, c["divd_size"], variant)) == c["out"], (kind, c["n"])


def test_pow_and_decimal_golden(ctx, golden):
    for c in golden["pow"]:
        p = ctx.pow(np.array([c["base"]], dtype=np.uint64), c["e"])
        assert digest(p) == c["out"]
        assert sdig(ctx.to_dec(p)) == c["dec"]
    for c in golden["to_dec"]:
        assert sdig(ctx.to_dec(limbs(c["seed"], c["n"]))) == c["out"]


@pytest.mark.parametrize("idx", [0, 1])
def test_pi_golden(ctx, golden, idx):
    c = golden["pi"][idx]
    assert sdig(ctx.pi_dec(c["terms"], c["acc"], c["digits"])) == c["out"]


@pytest.mark.parametrize("idx", [0, 1])
def test_e_golden(ctx, golden, idx):
    c = golden["e"][idx]
    assert sdig(ctx.e_dec(c["terms"], c["digits"])) == c["out"]


def test_cpp_dropin_program(golden, tmp_path):
    """The C++ surface compiles unchanged-style user code and prints the
    reference's 2^65536 (its demo program's output), consistent q and r,
    2000! and decimal / hex round trips."""
    import natural_number_gb300 as nn
    nn.lib()
    exe = tmp_path / "demo"
    subprocess.check_call(["g++", "-O2", "-std=c++20", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "natural_demo.cpp"), "-o", str(exe),
                           "-L", os.path.dirname(nn.LIB_PATH), "-lnatural_gb300",
                           "-Wl,-rpath," + os.path.dirname(nn.LIB_PATH)])
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300, check=True).stdout.split("\n")
    want = [c for c in golden["pow"] if c["base"] == 2 and c["e"] == 65536][0]["dec"]
    assert sdig(out[0]) == want
    assert out[3] == "ok"
    A, B = 3**4000, 7**1500 + 12345
    assert int(out[1], 16) == A // B and int(out[2]) == A % B
    import math
    assert int(out[4]) == math.factorial(2000)
    assert out[5] == "dec ok" and out[6] == "hex ok"
    ns = list(range(41)) + [63, 64, 100, 127, 128, 255, 1000]
    assert [int(v) for v in out[7].split()] == [math.factorial(n) for n in ns]
    strs = ["0", "7", "18446744073709551615", "18446744073709551616", "000123", "",
            "340282366920938463463374607431768211456"]
    assert [int(v, 16) for v in out[8].split()] == [int(t) if t else 0 for t in strs]


# Divisions on which the reference's own Newton division aborts
# (natural.h:670-676); the product takes its exact Newton division instead.
REFERENCE_ABORTS = [(5046, 7406, 5047, 3703), (19141, 4406, 19142, 2203)]


def test_divisions_the_reference_cannot_do(ctx):
    from oracle import to_int
    for sa, na, sb, nb in REFERENCE_ABORTS:
        a, b = limbs(sa, na), limbs(sb, nb)
        q, r = ctx.div(a, b)
        A, B = to_int(a), to_int(b)
        assert to_int(q) == A // B and to_int(r) == A % B


@pytest.mark.parametrize("seed", range(3))
def test_random_2n_by_n_divisions(ctx, seed):
    """Random 2n-by-n divisions (the served division shape) against Python integers."""
    from oracle import to_int
    from natural_number_gb300.synth import log_uniform_sizes
    for k, n in enumerate(log_uniform_sizes(100 + seed, 40, 1, 13)):
        n = max(2, int(n))
        a, b = limbs(seed * 10000 + 2 * k, 2 * n), limbs(seed * 10000 + 2 * k + 1, n)
        q, r = ctx.div(a, b)
        A, B = to_int(a), to_int(b)
        assert to_int(q) == A // B and to_int(r) == A % B, n


@pytest.mark.parametrize("idx", [0, 1, 2, 3])
def test_pi_levels_golden(ctx, golden, idx):
    """pi with the level-by-level batched trees equals the reference's digits;
    host_below=8 sends all but the smallest products to the GPU."""
    c = golden["pi"][idx]
    s, t = ctx.pi_dec_levels(c["terms"], c["acc"], c["digits"], host_below=8 if idx < 2 else 128)
    assert sdig(s) == c["out"]
    assert t["gpu_products"] > 0


@pytest.mark.parametrize("idx", [0, 1, 2, 3])
def test_e_levels_golden(ctx, golden, idx):
    c = golden["e"][idx]
    s, t = ctx.e_dec_levels(c["terms"], c["digits"], host_below=8 if idx < 2 else 128)
    assert sdig(s) == c["out"]


def test_to_dec_levels_golden(ctx, golden):
    for c in golden["to_dec"]:
        assert sdig(ctx.to_dec_levels(limbs(c["seed"], c["n"]), host_below=4)) == c["out"]
    for c in golden["pow"]:
        p = ctx.pow(np.array([c["base"]], dtype=np.uint64), c["e"])
        assert sdig(ctx.to_dec_levels(p, host_below=4)) == c["dec"]


@pytest.mark.parametrize("host_below", [4, 64, 256])
def test_to_dec_levels_edges_vs_python(ctx, host_below):
    """Decimal strings from the split levels and the device leaves against
    Python's str(): random values of 1 to 5000 limbs, powers of ten and their
    neighbours at the 18-digit group and split-power boundaries (values whose
    low groups are all zero, first nodes with leading zeros in their field),
    powers of two and all-ones limbs."""
    import sys
    old = sys.get_int_max_str_digits()
    sys.set_int_max_str_digits(0)
    try:
        vals = []
        for k, n in enumerate([1, 2, 3, 5, 17, 64, 129, 300, 1000, 5000]):
            vals.append(_int(limbs(900 + k, n)))
        for e in [18, 19, 35, 36, 37, 72, 144, 288, 576, 1152, 2304, 4608, 9216, 20000]:
            vals += [10 ** e - 1, 10 ** e, 10 ** e + 1, 10 ** e * 7 + 3]
        vals += [2 ** 64, 2 ** 64 - 1, 2 ** 4096, 2 ** 20000 - 1, 10 ** 5000 * (2 ** 64 - 1)]
        for v in vals:
            got = ctx.to_dec_levels(_limbs_of(v), host_below=host_below)
            assert got == str(v), (v.bit_length(), host_below)
    finally:
        sys.set_int_max_str_digits(old)


def test_to_dec_levels_long_nodes_vs_recursive(ctx):
    """Values of 2^17 to 2^18 limbs, whose top split levels have nodes of
    2^16 limbs and more (corrected by multiword scans rather than one warp a
    node): all-nines and powers of ten at a split power, and random limbs,
    against the recursive conversion (natural's own to_string)."""
    import sys
    old = sys.get_int_max_str_digits()
    sys.set_int_max_str_digits(0)
    try:
        e = 18 * 2 ** 18
        vals = [10 ** e - 1, 10 ** e, 3 * 10 ** e - 1]
        vals = [_limbs_of(v) for v in vals] + [limbs(4242, 1 << 18), limbs(4243, (1 << 17) + 12345)]
        for x in vals:
            assert ctx.to_dec_levels(x) == ctx.to_dec(x), x.size
    finally:
        sys.set_int_max_str_digits(old)


@pytest.mark.parametrize("kind", ["pi", "e"])
def test_levels_1e7_and_1e8_digits(ctx, golden, kind):
    """pi and e to 10^7 and 10^8 digits (the reference's recipes with 2^20 /
    2^23 and 2^21 / 2^24 terms) with the default split between host subtrees
    and GPU levels: SHA-256 of the digit strings equal to the reference's."""
    import hashlib
    for c in (golden[kind][4], golden["big_" + kind][0]):
        if kind == "pi":
            s, _ = ctx.pi_dec_levels(c["terms"], c["acc"], c["digits"])
        else:
            s, _ = ctx.e_dec_levels(c["terms"], c["digits"])
        assert len(s) == c["out"]["len"]
        assert hashlib.sha256(s.encode()).hexdigest() == c["out"]["sha256"]
        del s


def _int(x):
    return int.from_bytes(np.ascontiguousarray(x, dtype="<u8").tobytes(), "little")


def _limbs_of(v, n=None):
    n = n or max(1, (v.bit_length() + 63) // 64)
    return np.frombuffer(v.to_bytes(8 * n, "little"), dtype="<u8").astype(np.uint64)


def _check_divmod(ctx, x, y, q, r):
    """q, r = divmod(x, y): exactly by Python for small operands, else by
    q*y + r == x with the GPU product (tested on its own) and r < y."""
    Q, R = _int(q), _int(r)
    if x.bit_length() <= 64 * 20000:
        assert Q == x // y and R == x % y
    else:
        assert R < y
        assert _int(ctx.mul(q, _limbs_of(y))) + R == x


@pytest.mark.parametrize("na,nb", [(2048, 1024), (5000, 1024), (100000, 3000), (1 << 18, 1 << 17), (3000, 2999),
                                   ((1 << 16) + 5, 1030), (1024, 1024), (4000, 33), (70, 5)])
def test_device_division_vs_python(ctx, na, nb):
    """The division with every step on the GPU (nn_divmod_host, nn_div):
    quotient and remainder as Python's for short and long quotients,
    power-of-two, all-ones and near-multiple divisors."""
    import torch
    a, b = limbs(na * 7 + 1, na), limbs(nb * 11 + 3, nb)
    A, Bv = _int(a), _int(b)
    cases = [(A, Bv), (A, 1 << (64 * nb - 1)), (A, (1 << (64 * nb)) - 1), (A, Bv | 1)]
    if na <= 20000:  # exact multiples and one below need Python products of the full size
        cases += [(Bv * (A >> (64 * nb)), Bv), (Bv * (A >> (64 * nb)) - 1, Bv)]
    for x, y in cases:
        if x < 0:
            continue
        xa, ya = _limbs_of(x), _limbs_of(y)
        if xa.size < ya.size:
            continue
        q, r = ctx.divmod(xa, ya)
        _check_divmod(ctx, x, y, q, r)
    # device pointers
    dq = torch.zeros(na - nb + 1, dtype=torch.uint64, device="cuda")
    dr = torch.zeros(nb, dtype=torch.uint64, device="cuda")
    ctx.div_device(dq, dr, to_dev_np(a), to_dev_np(b))
    _check_divmod(ctx, A, Bv, dq.cpu().numpy(), dr.cpu().numpy())


def to_dev_np(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).to("cuda")


def test_device_division_on_reference_abort_inputs(ctx):
    """The GPU division also handles the inputs on which the reference's own
    division aborts, and large 2n-by-n cases."""
    for sa, na, sb, nb in REFERENCE_ABORTS + [(7, 9000, 8, 4500), (9, 300000, 10, 150000)]:
        a, b = limbs(sa, na), limbs(sb, nb)
        q, r = ctx.divmod(a, b)
        _check_divmod(ctx, _int(a), _int(b), q, r)
