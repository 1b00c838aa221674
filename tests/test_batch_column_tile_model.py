"""The index arithmetic of the batch kernel's base-case items
(natural_number_gb300/csrc/batch.cu: column_tile_sums, SmemSumsProducer),
restated in Python and checked on the CPU: for every tile of a product, the
positions whose column sums the item stores cover every position the carry
scan of that tile reads below the product's length (its 2048 positions and
the 8 before them), stay within the shared array of 3 x 2056 words, and the
eight-lane groups' rounds visit each stored position exactly once.  The
column sums themselves, computed eight lanes a position, equal the
schoolbook columns of the product."""
import random

import pytest

SCAN_TILE = 256 * 8
SCAN_E = 8
COLUMN_TILE_WORDS = SCAN_TILE + SCAN_E
LANES, GROUPS = 8, 256 // 8


def tile_plan(size, tile):
    """(first, npos, rounds) of column_tile_sums."""
    first = tile * SCAN_TILE - SCAN_E
    end = min(size, (tile + 1) * SCAN_TILE)
    npos = end - first
    return first, npos, (npos + GROUPS - 1) // GROUPS


def scan_reads(size, tile):
    """Positions scan_tile asks the producer for that lie below the total
    (the producer answers zero at and above it without reading)."""
    own = range(tile * SCAN_TILE, (tile + 1) * SCAN_TILE)
    before = range(tile * SCAN_TILE - SCAN_E, tile * SCAN_TILE) if tile else range(0)
    return [k for k in list(before) + list(own) if k < size]


@pytest.mark.parametrize("size", [2, 3, 9, 100, 2047, 2048, 2049, 2056, 2057, 4095, 4096, 4097, 6000, 14000])
def test_stored_positions_cover_the_scan(size):
    tiles = (size + SCAN_TILE - 1) // SCAN_TILE
    for tile in range(tiles):
        first, npos, rounds = tile_plan(size, tile)
        assert 0 < npos <= COLUMN_TILE_WORDS
        stored = []
        for r in range(rounds):
            for g in range(GROUPS):
                q = r * GROUPS + g
                if q < npos:
                    stored.append(first + q)
        assert len(stored) == len(set(stored)) == npos
        lo, hi = first, first + npos
        for k in scan_reads(size, tile):
            assert lo <= k < hi, (size, tile, k)
            assert 0 <= k - first < COLUMN_TILE_WORDS  # the producer's index, mod 2^64 for tile 0


def column_sum_by_lanes(a, b, k):
    """One position's sum as the eight lanes form it, then their reduction."""
    na, nb = len(a), len(b)
    if k + 1 >= na + nb:
        return 0
    lo = k - nb + 1 if k >= nb else 0
    hi = k if k < na - 1 else na - 1
    lanes = [sum(a[i] * b[k - i] for i in range(lo + j, hi + 1, LANES)) for j in range(LANES)]
    d = LANES // 2
    while d >= 1:  # __shfl_down_sync(..., d, 8): lane j adds lane j + d
        lanes = [lanes[j] + (lanes[j + d] if j + d < LANES else 0) for j in range(LANES)]
        d //= 2
    return lanes[0]


def test_column_sums_by_lanes_equal_schoolbook_columns():
    rng = random.Random(5)
    M = (1 << 64) - 1
    for na, nb in [(1, 1), (1, 9), (7, 3), (33, 31), (100, 80), (300, 9)]:
        a = [rng.choice([M, rng.randrange(1 << 64)]) for _ in range(na)]
        b = [rng.choice([M, rng.randrange(1 << 64)]) for _ in range(nb)]
        for k in range(na + nb):
            want = sum(a[i] * b[k - i] for i in range(na) if 0 <= k - i < nb)
            got = column_sum_by_lanes(a, b, k)
            assert got == want and got < 1 << 192
