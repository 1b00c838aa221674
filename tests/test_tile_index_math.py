"""The shared-memory index arithmetic of the tiled NTT passes
(natural_number_gb300/csrc/ntt_tiles.cuh: pad16, level_group, tile_forward,
tile_inverse), restated in Python and checked on the CPU for every tile shape
the passes use: tile widths C = 2, 16, 32, 64, 128, up to 2^11 rows, groups
starting at any skipped level.  level_group reads row m of a unit at
pad16(x0) + off(m); that is only the padded address of x0 + m*S when the
identity below holds, and every index must stay inside the padded tile."""
import pytest

THREADS = 256


def pad16(x):
    return x + ((x >> 5) << 1)


def tile_words(nel):
    return (nel + nel // 16 + 3) & ~1


def group_cap(C, R):
    k = min(R, 3)
    while k > 1 and (C << (R - k)) < THREADS:
        k -= 1
    return k


def forward_groups(C, R, l0):
    cap = group_cap(C, R)
    n = (R - l0 + cap - 1) // cap
    out, l = [], l0
    for g in range(n):
        k = (R - l + (n - g) - 1) // (n - g)
        out.append((l, k))
        l += k
    assert l == R
    return out


def inverse_groups(C, R, l_stop):
    cap = group_cap(C, R)
    n = (R - l_stop + cap - 1) // cap
    out, l = [], R
    for g in range(n):
        k = (l - l_stop + (n - g) - 1) // (n - g)
        l -= k
        out.append((l, k))
    assert l == l_stop
    return out


def check_group(C, R, l, K):
    nsub = R - l - K
    units = C << (R - K)
    S = C << nsub
    tmask = (1 << nsub) - 1
    nel = C << R
    limit = tile_words(nel)
    seen = set()
    for u in range(units):
        i = u & (C - 1)
        v = u // C
        rb = v >> nsub
        row0 = (rb << (R - l)) + (v & tmask)
        x0 = row0 * C + i
        base = pad16(x0)
        for m in range(1 << K):
            off = m * S + (((m * S) >> 5) << 1)
            assert pad16(x0 + m * S) == base + off, (C, R, l, K, u, m)
            assert base + off < limit
            seen.add(x0 + m * S)
    assert seen == set(range(nel))  # each group touches every element once


@pytest.mark.parametrize("C", [2, 16, 32, 64, 128])
def test_level_groups_index_identity(C):
    for R in range(1, 12):
        if (C << R) > 8192:
            continue
        shapes = set()
        for skip in range(R):
            shapes.update(forward_groups(C, R, skip))
            shapes.update(inverse_groups(C, R, skip))
        for l, K in shapes:
            check_group(C, R, l, K)


def test_radix16_groups_of_11_level_contiguous_tiles():
    """The compile-time schedule of 11-level contiguous tiles (C = 2) runs
    4 + 4 + 3 levels forward and 4 + 4 + 3 back (tile_forward_ct /
    tile_inverse_ct): 16-row units, one per thread."""
    C, R = 2, 11
    fwd, inv, l = [], [], 0
    n = 3
    for g in range(n):
        k = (R - l + (n - g) - 1) // (n - g)
        fwd.append((l, k))
        l += k
    l = R
    for g in range(n):
        k = (l + (n - g) - 1) // (n - g)
        l -= k
        inv.append((l, k))
    assert fwd == [(0, 4), (4, 4), (8, 3)] and inv == [(7, 4), (3, 4), (0, 3)]
    for l, K in fwd + inv:
        assert (C << (R - K)) >= THREADS
        check_group(C, R, l, K)


def test_wide_tile_loads_aligned():
    """Pass loads copy pairs (idx, idx+1) with 16-byte copies: both the global
    position and the padded shared index must be even."""
    for C, lgc in [(2, 1), (16, 4), (32, 5), (64, 6), (128, 7)]:
        for R in range(1, 12):
            nel = C << R
            if nel > 8192:
                continue
            for lg_s in (lgc, lgc + 1, lgc + 5):
                if (1 << lg_s) < C:
                    continue
                tiles_per_sb = (1 << lg_s) // C
                for tile in (0, 1, tiles_per_sb - 1, tiles_per_sb, 3 * tiles_per_sb + 1):
                    ksb, t = divmod(tile, tiles_per_sb)
                    base = (ksb << (lg_s + R)) + t * C
                    for idx in range(0, nel, 2):
                        pos = base + ((idx >> lgc) << lg_s) + (idx & (C - 1))
                        assert pos % 2 == 0 and pad16(idx) % 2 == 0
