"""The batch's split of unbalanced products (natural_number_gb300/csrc/
engine.cpp: batch_split; scan_tiles.cuh: PieceCrtProducer), restated in
Python and checked on the CPU with exact integers: the pieces' products,
summed coefficient by coefficient as the CRT scan sums them, give the whole
product; every piece product fits its transform; eight positions starting at
a multiple of 8 lie in one piece (the scan's vector loads)."""
import random

B = 1 << 64
RATE = [1.0, 1.0, 1.0, 1.0, 1.2, 1.4, 1.7, 2.0, 2.3, 2.57, 4.77, 6.94, 7.51, 6.9, 6.9, 6.66, 6.39, 6.08, 5.63,
        5.66, 5.65]


def rate(s):
    return RATE[s] if s < len(RATE) else 5.0


def ntt_scale(na, nb):
    s = 2
    while (1 << s) < na + nb - 1:
        s += 1
    return s


def batch_split(nx, ny, s):
    best = 3.0 * (1 << s) / rate(s)
    s_best, k, P = s, nx, 1
    for s2 in range(s - 1, 1, -1):
        L2 = 1 << s2
        if L2 + 1 < 2 * ny:
            break
        kk = (L2 - ny + 1) & ~7
        if kk < ny or kk >= nx:
            continue
        pieces = (nx + kk - 1) // kk
        cost = (2.0 * pieces + 1.0) * L2 / rate(s2)
        if cost < 0.95 * best:
            best, s_best, k, P = cost, s2, kk, pieces
    return s_best, k, P


def coeffs(x, y):
    out = [0] * (len(x) + len(y) - 1)
    for u, xv in enumerate(x):
        if xv:
            for v, yv in enumerate(y):
                out[u + v] += xv * yv
    return out


def value(limbs):
    return sum(v << (64 * i) for i, v in enumerate(limbs))


def check(nx, ny, rng):
    s = ntt_scale(nx, ny)
    s2, k, P = batch_split(nx, ny, s)
    x = [rng.getrandbits(64) for _ in range(nx)]
    y = [rng.getrandbits(64) for _ in range(ny)]
    if P == 1:
        assert (s2, k) == (s, nx)
        return 0
    L2 = 1 << s2
    assert k % 8 == 0 and ny <= k < nx and k + ny - 1 <= L2 and (P - 1) * k < nx <= P * k
    pieces = [coeffs(x[i * k:(i + 1) * k], y) for i in range(P)]
    assert all(len(c) <= L2 for c in pieces)  # no wrap in any piece's transform
    count = nx + ny - 1

    def piece_of(j):
        return min(j // k, P - 1)

    def at(i, r):
        c = pieces[i]
        assert r < L2
        return c[r] if r < len(c) else 0

    total = 0
    for j in range(count):
        i = piece_of(j)
        r = j - i * k
        v = at(i, r)
        if i > 0 and r + 1 < ny:
            v += at(i - 1, r + k)
        assert v < 1 << 160
        total += v << (64 * j)
    assert total == value(x) * value(y)
    for k0 in range(0, count - 7, 8):
        assert len({piece_of(k0 + e) for e in range(8)}) == 1
    return P


def test_split_pieces_sum_to_product():
    rng = random.Random(5)
    split = 0
    cases = [(5000, 128), (2000, 20), (3000, 50), (1500, 100), (800, 30), (4096, 64), (2100, 129), (1200, 9),
             (6000, 300), (1 << 12, 200)]
    for nx, ny in cases:
        split += check(nx, ny, rng) > 1
    assert split >= 6


def test_split_choices_over_sizes():
    """Only the planner's constraints, over many sizes (no products)."""
    for nx in [384, 1000, 5000, 1 << 14, 100000, 1 << 18, (1 << 18) + 3, 1 << 20]:
        for ny in [128, 129, 200, 384, 1000, 4096, 1 << 14, 1 << 16, 1 << 18]:
            if ny > nx:
                continue
            s = ntt_scale(nx, ny)
            s2, k, P = batch_split(nx, ny, s)
            if P > 1:
                assert s2 < s and k % 8 == 0 and ny <= k < nx and k + ny - 1 <= 1 << s2
                assert (P - 1) * k < nx <= P * k
