"""The carries between scan tiles (natural_number_gb300/csrc/carry.cu:
tile_carry_kernel and carry_fix_kernel), restated in Python and checked on
the CPU against plain sequential addition.

Every tile first runs with carry-in 0 and records a generate bit (carry out
for carry-in 0) and a propagate bit (all limbs ones, so a carry-in passes
straight through).  One CTA of 1024 threads then takes the tiles in chunks of
32 per thread, folds each thread's tiles into a map carry-in -> carry-out,
composes the maps with a Hillis-Steele scan, and walks the tiles again to
give every tile its carry-in; chunks, and the ranges of one scan, chain
their carries.  Finally each tile with
carry-in 1 adds it at its first limb, rippling while limbs wrap."""
import random

import pytest

THREADS = 1024
PER = 32
CHUNK = THREADS * PER
M = (1 << 64) - 1


def tile_carries(flags, t0, t1, chain):
    """tile_carry_kernel: returns the per-tile carry-ins and the new chain."""
    out = {}
    carry = chain if t0 > 0 else 0
    for c0 in range(t0, t1, CHUNK):
        n = min(CHUNK, t1 - c0)
        sb = [flags[c0 + k] if k < n else 2 for k in range(CHUNK)]  # padding propagates
        f = []
        for j in range(THREADS):
            f0, f1 = 0, 1
            for v in sb[j * PER:(j + 1) * PER]:
                g, p = v & 1, (v >> 1) & 1
                f0, f1 = g | (p & f0), g | (p & f1)
            f.append((f0, f1))
        d = 1
        while d < THREADS:  # inclusive scan of the maps, earlier map applied first
            old = list(f)
            for j in range(d, THREADS):
                e0, e1 = old[j - d]
                f0, f1 = old[j]
                f[j] = (f1 if e0 else f0, f1 if e1 else f0)
            d <<= 1
        for j in range(THREADS):
            c = carry if j == 0 else (f[j - 1][1] if carry else f[j - 1][0])
            for i in range(PER):
                k = j * PER + i
                v = sb[k]
                if k < n:
                    out[c0 + k] = c
                c = (v & 1) | ((v >> 1) & c)
            if j == THREADS - 1:
                last = c
        carry = last
    return out, carry


def run(tile_values, tile_limbs, ranges):
    """Limb arrays per tile (values with carry-in 0 as step 1 leaves them,
    and each tile's carry out for carry-in 0) -> final limbs."""
    limbs, flags = [], []
    for vals, cout in tile_values:
        assert len(vals) == tile_limbs
        allones = all(v == M for v in vals)
        assert not (cout and allones)
        flags.append(cout | (int(allones) << 1))
        limbs.extend(vals)
    chain = 0
    cins = {}
    for t0, t1 in ranges:
        c, chain = tile_carries(flags, t0, t1, chain)
        cins.update(c)
    for t, cin in cins.items():  # carry_fix_kernel
        if cin:
            for k in range(t * tile_limbs, (t + 1) * tile_limbs):
                limbs[k] = (limbs[k] + 1) & M
                if limbs[k]:
                    break
    return limbs


def sequential(tile_values, tile_limbs):
    total, shift = 0, 0
    for vals, cout in tile_values:
        v = sum(x << (64 * i) for i, x in enumerate(vals)) + (cout << (64 * tile_limbs))
        total += v << shift
        shift += 64 * tile_limbs
    return [(total >> (64 * i)) & M for i in range(len(tile_values) * tile_limbs)]


def make(n_tiles, tile_limbs, rng, p_ones=0.3):
    out = []
    for _ in range(n_tiles):
        r = rng.random()
        if r < p_ones:  # all ones: propagates
            out.append(([M] * tile_limbs, 0))
        elif r < p_ones + 0.1:  # ones up to a zero limb near the end
            vals = [M] * tile_limbs
            vals[-1] = 0
            out.append((vals, rng.randrange(2)))
        else:
            out.append(([rng.getrandbits(64) for _ in range(tile_limbs)], rng.randrange(2)))
    return out


@pytest.mark.parametrize("n_tiles", [1, 2, 7, 1023, 1025, 32768, 40000])
def test_tile_carries_match_sequential_addition(n_tiles):
    rng = random.Random(n_tiles)
    tv = make(n_tiles, 3, rng)
    assert run(tv, 3, [(0, n_tiles)]) == sequential(tv, 3)


def test_ranges_chain_their_carries():
    rng = random.Random(5)
    n = 36000
    tv = make(n, 2, rng, p_ones=0.6)
    cuts = [0, 1, 700, 701, 2048, 34000, n]
    assert run(tv, 2, list(zip(cuts, cuts[1:]))) == sequential(tv, 2)


def test_long_run_of_ones_ends_in_a_carry():
    # every tile all ones but the first generates: the carry runs through all
    tv = [([5, 7], 1)] + [([M, M], 0)] * 2000
    assert run(tv, 2, [(0, len(tv))]) == sequential(tv, 2)
