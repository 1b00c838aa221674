"""GPU parity: the sm_103a NTT path against the oracle and the reference's
golden vectors, through the C ABI.  Integer work, so every check is bit-exact."""
import numpy as np
import pytest

from gpu_util import P, digest, empty_dev, mod_checks, normalize, to_dev, to_host
from natural_number_gb300.synth import limbs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import natural_number_gb300 as nn
    c = nn.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("s,n", [(3, 2), (3, 4), (4, 7), (10, 300), (10, 1000), (12, 2048), (12, 3000),
                                 (14, 16384), (15, 9000), (21, 1 << 20), (21, (1 << 20) + 12345), (23, 3 << 21)])
def test_forward_residues_canonical(ctx, oracle, s, n):
    """Residues after load + forward NTT equal the oracle's (the reference's
    transform: same CRT-tree order and twiddles) modulo each prime, and stay in
    the lazy ranges the next stage accepts: [0, 4p) for p0 and p1 (4p < 2^64),
    [0, 2p) for p2."""
    a = limbs(1000 + s * 7 + n, n)
    t = ctx.transform().forward(to_dev(a), s)
    out = empty_dev(3 << s)
    t.residues(out)
    got = to_host(out).reshape(3, 1 << s)
    want = oracle.ntt_forward(a, s)
    for i in range(3):
        p = np.uint64(P[i])
        assert int(got[i].max()) < (4 if i < 2 else 2) * P[i]
        if not np.array_equal(got[i] % p, want[i] % p):
            bad = np.nonzero(got[i] % p != want[i] % p)[0]
            pytest.fail(f"prime {i}: {bad.size} mismatches, first at {bad[:5]}")


def test_forward_golden_canonical(ctx, golden):
    for c in golden["ntt_forward"]:
        s = c["scale"]
        t = ctx.transform().forward(to_dev(limbs(c["seed"], c["n"])), s)
        out = empty_dev(3 << s)
        t.residues(out)
        got = to_host(out).reshape(3, 1 << s)
        canon = np.stack([got[i] % np.uint64(P[i]) for i in range(3)])
        assert digest(canon.ravel()) == c["canonical"]


def test_ntt_raw_golden_including_wrap(ctx, golden):
    for c in golden["ntt_raw"]:
        a, b = limbs(c["seed_a"], c["na"]), limbs(c["seed_b"], c["nb"])
        s, size = c["scale"], c["size"]
        out = empty_dev(max(size, 1 << s))
        w = ctx.ntt_mul_device(out, to_dev(a), to_dev(b), s, size)
        assert w == c["out"]["n"]
        assert digest(to_host(out, w)) == c["out"], c


@pytest.mark.parametrize("seed", range(6))
def test_ntt_raw_random_wrap_vs_oracle(ctx, oracle, seed):
    rng = np.random.default_rng(seed)
    s = int(rng.integers(9, 15))
    L = 1 << s
    na = int(rng.integers(L // 3, L + 1))
    nb = int(rng.integers(L // 3, L + 1))
    size = int(rng.choice([na + nb, L + 1, L + 2, L + 7, na + nb + 5]))
    a, b = limbs(seed * 31 + 1, na), limbs(seed * 31 + 2, nb)
    if seed % 2:  # saturated limbs stress the carry chain
        a[:] = np.uint64(2**64 - 1)
        b[: nb // 2] = np.uint64(2**64 - 1)
    out = empty_dev(max(size, L))
    w = ctx.ntt_mul_device(out, to_dev(a), to_dev(b), s, size)
    want = oracle.ntt_mul_raw(a, b, s, size)
    assert w == want.size
    assert np.array_equal(to_host(out, w), want)


def test_mul_golden(ctx, golden):
    for c in golden["mul"]:
        a, b = limbs(c["seed_a"], c["na"]), limbs(c["seed_b"], c["nb"])
        assert digest(ctx.mul(a, b)) == c["out"], (c["na"], c["nb"])


def test_sqr_golden(ctx, golden):
    for c in golden["sqr"]:
        assert digest(ctx.sqr(limbs(c["seed"], c["n"]))) == c["out"], c["n"]


@pytest.mark.parametrize("na,nb", [(1, 1), (1, 5), (7, 1), (31, 33), (383, 5000), (384, 384), (385, 4000),
                                   (1000, 999), (4097, 4095), (70001, 65536), (100000, 50001), (262145, 131072)])
def test_mul_vs_oracle(ctx, oracle, na, nb):
    a, b = limbs(na * 3 + 1, na), limbs(nb * 5 + 2, nb)
    assert np.array_equal(ctx.mul(a, b), oracle.mul(a, b))


def test_mul_edge_values(ctx, oracle):
    cases = [([0], [0]), ([0], list(range(1, 600))), ([2**64 - 1] * 500, [2**64 - 1] * 700),
             ([1], [2**64 - 1] * 3), ([0, 0, 1], [0, 1]), ([2**64 - 1] * 4096, [2**64 - 1] * 4096)]
    for a, b in cases:
        a = np.array(a, dtype=np.uint64)
        b = np.array(b, dtype=np.uint64)
        assert np.array_equal(normalize(ctx.mul(a, b)), normalize(oracle.mul(a, b)))
    for n in (1, 47, 383, 384, 5000):
        a = np.full(n, 2**64 - 1, dtype=np.uint64)
        assert np.array_equal(ctx.sqr(a), oracle.sqr(a))


def test_device_api_matches_host_api(ctx, oracle):
    a, b = limbs(11, 50000), limbs(12, 30000)
    out = empty_dev(80000)
    ctx.mul_device(out, to_dev(a), to_dev(b))
    assert np.array_equal(normalize(to_host(out)), oracle.mul(a, b))
    out2 = empty_dev(100000)
    ctx.sqr_device(out2, to_dev(a))
    assert np.array_equal(normalize(to_host(out2)), oracle.sqr(a))


def test_config1_plain_multiply_bit_exact(ctx, oracle):
    """2^20 x 2^20 limbs, seeded, against the oracle's operator*."""
    n = 1 << 20
    a, b = limbs(1, n), limbs(2, n)
    got = ctx.mul(a, b)
    assert got.size == 2 * n
    assert np.array_equal(got, oracle.mul(a, b))


def test_config2_large_multiply_and_square(ctx, golden):
    """2^27-limb operands: digest of the reference's own product/square when
    the big fixtures exist, plus size-independent modular checks."""
    n = 1 << 27
    a, b = limbs(1000 + n, n), limbs(7777 + n, n)
    da, db = to_dev(a), to_dev(b)
    out = empty_dev(2 * n)
    ctx.mul_device(out, da, db)
    prod = to_host(out)
    ma, mb, mp = mod_checks(a), mod_checks(b), mod_checks(prod)
    assert mp[0] == ma[0] * mb[0] % (2**64 - 1)
    assert mp[1] == ma[1] * mb[1] % (2**64 + 1)
    for c in golden.get("big_mul", []):
        if c["na"] == n:
            assert digest(normalize(prod)) == c["out"]
    del prod
    ctx.sqr_device(out, da)
    sq = to_host(out)
    ms = mod_checks(sq)
    assert ms[0] == ma[0] * ma[0] % (2**64 - 1)
    assert ms[1] == ma[1] * ma[1] % (2**64 + 1)
    for c in golden.get("big_sqr", []):
        if c["n"] == n:
            assert digest(normalize(sq)) == c["out"]


@pytest.mark.parametrize("na,nb", [(1 << 16, 1 << 16), (50000, 3000), (200, 150), (70000, 65536), (300001, 200003),
                                   (900001, 800003)])
def test_mul_host_page_locked(ctx, oracle, na, nb):
    """Host products on page-locked operands and result (as the benchmark's
    end-to-end leg uses them), for the balanced NTT, split and base-case
    paths, in both operand orders; and the same product from pageable arrays.
    The balanced products copy the longer operand a column range at a time
    while the first pass runs; odd lengths leave a partial last row."""
    import torch
    a, b = limbs(31 + na, na), limbs(37 + nb, nb)
    pa = torch.from_numpy(a).pin_memory().numpy()
    pb = torch.from_numpy(b).pin_memory().numpy()
    po = torch.zeros(na + nb, dtype=torch.uint64).pin_memory().numpy()
    want = oracle.mul(a, b)
    got = ctx.mul(pa, pb, out=po)
    assert np.array_equal(got, want)
    got = ctx.mul(pb, pa, out=po)  # shorter operand first
    assert np.array_equal(got, want)
    assert np.array_equal(ctx.mul(a, b), want)  # pageable
    # operands one limb into their host buffers (8-byte aligned views)
    va, vb = np.empty(na + 1, dtype=np.uint64), np.empty(nb + 1, dtype=np.uint64)
    va[1:], vb[1:] = a, b
    assert np.array_equal(ctx.mul(va[1:], vb[1:]), want)


@pytest.mark.parametrize("na,nb", [(1 << 25, 1000), (1 << 25, 383), ((1 << 24) + 12345, (1 << 20) + 7),
                                   (3 << 23, 1 << 23), ((1 << 26) - 1, (1 << 26) - 1)])
def test_large_unbalanced_products_mod_checks(ctx, na, nb):
    """Large products through every dispatch path (schoolbook below 384 limbs,
    the reference's unbalanced split, balanced NTT just below a scale
    boundary), checked by the product's residues mod 2^64 - 1 and 2^64 + 1."""
    a, b = limbs(101 + na, na), limbs(103 + nb, nb)
    out = empty_dev(na + nb)
    ctx.mul_device(out, to_dev(a), to_dev(b))
    prod = to_host(out)
    ma, mb, mp = mod_checks(a), mod_checks(b), mod_checks(prod)
    assert mp[0] == ma[0] * mb[0] % (2**64 - 1)
    assert mp[1] == ma[1] * mb[1] % (2**64 + 1)


@pytest.mark.parametrize("n", [(1 << 21) + 3, 3 << 20])
def test_carry_chains_across_many_scan_tiles(ctx, n):
    """(B^n - 1)^2 = B^2n - 2 B^n + 1: its upper half is all-ones limbs, so
    the CRT scan's tile carries propagate through thousands of tiles (scans
    of more than 1024 tiles resolve them in separate steps rather than by the
    lookback).  Through the device path and the host path, whose scan runs
    in ranges of tiles with the copy-back of each range queued behind it."""
    M = np.uint64(0xFFFFFFFFFFFFFFFF)
    a = np.full(n, M, dtype=np.uint64)
    want = np.concatenate([[np.uint64(1)], np.zeros(n - 1, dtype=np.uint64), [M - np.uint64(1)],
                           np.full(n - 1, M, dtype=np.uint64)])
    out = empty_dev(2 * n)
    ctx.mul_device(out, to_dev(a), to_dev(a))
    assert np.array_equal(to_host(out), want)
    assert np.array_equal(ctx.mul(a, a), want)
    assert np.array_equal(ctx.sqr(a), want)


def test_multi_step_scan_vs_oracle(ctx, oracle):
    """A 2^21 x 2^21-limb product (2048 scan tiles, past the lookback's 1024)
    against the oracle, device and host paths."""
    n = 1 << 21
    a, b = limbs(61, n), limbs(62, n)
    want = oracle.mul(a, b)
    out = empty_dev(2 * n)
    ctx.mul_device(out, to_dev(a), to_dev(b))
    assert np.array_equal(to_host(out), want)
    assert np.array_equal(ctx.mul(a, b), want)


@pytest.mark.parametrize("na,nb", [(300, 200), (383, 383), (5000, 3001), (1 << 16, 1 << 16), (200000, 70001)])
def test_products_on_8_byte_aligned_buffers(ctx, oracle, na, nb):
    """Operands and products one limb into their buffers (8-byte, not 16-byte,
    aligned): the first pass's limb loads take their scalar path and the
    carry scan its scalar stores, and the results equal the oracle's."""
    a, b = limbs(8000 + na, na), limbs(9000 + nb, nb)
    da, db = empty_dev(na + 1), empty_dev(nb + 1)
    da[1:] = to_dev(a)
    db[1:] = to_dev(b)
    out = empty_dev(na + nb + 1)
    ctx.mul_device(out[1:], da[1:], db[1:])
    assert np.array_equal(normalize(to_host(out)[1:]), oracle.mul(a, b))
    out2 = empty_dev(2 * na + 1)
    ctx.sqr_device(out2[1:], da[1:])
    assert np.array_equal(normalize(to_host(out2)[1:]), oracle.sqr(a))


def test_wrap_mode_on_8_byte_aligned_buffers(ctx, oracle):
    """The wrap-mode pipeline with operands and output one limb into their
    buffers, against the oracle."""
    s, size = 14, (1 << 14) + 9
    a, b = limbs(77, 12000), limbs(78, 9000)
    da, db, out = empty_dev(12001), empty_dev(9001), empty_dev((1 << s) + 1)
    da[1:] = to_dev(a)
    db[1:] = to_dev(b)
    w = ctx.ntt_mul_device(out[1:], da[1:], db[1:], s, size)
    assert np.array_equal(to_host(out)[1:1 + w], oracle.ntt_mul_raw(a, b, s, size))
