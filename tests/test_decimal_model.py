"""The arithmetic of the device's decimal output and batched sums
(natural_number_gb300/csrc/decimal.cu, carry.cu add_batch_kernel), restated
in Python and checked on the CPU against Python integers.

- Division by 10^18 with the normalised divisor 16 * 10^18 and the two-by-one
  step of Moller and Granlund (IEEE Trans. Computers 60(2), 2011,
  Algorithm 4), the remainder kept shifted by 4 bits.
- One warp a node: lane l reduces its segment of limbs to the map
  r -> (r * 2^(64 len) + segment) mod 10^18; a scan from the top lane down
  composes the maps; every lane then forms its quotient limbs from the
  remainder entering its segment.
- One warp a sum: a 32-limb step's carries are those of the integer sum
  G + (G | P) + carry-in over the lanes' generate and propagate bits; a
  difference adds the complement with a carry-in of 1; past the shorter
  operand the walk stops once nothing is pending.
- The split's correction (natural.h:962-965) and the 18-digit groups.
"""
import random

import pytest

M = (1 << 64) - 1
B = 1 << 64
D = 10**18
NORM = 4
DN = D << NORM
V = ((1 << 128) - 1) // DN - (1 << 64)  # the reciprocal, 64 bits
W = 32


def div_2by1(u1, u0):
    """(q, r) of (u1 * 2^64 + u0) / DN for u1 < DN (decimal.cu: div_2by1)."""
    p = V * u1
    p_lo, p_hi = p & M, p >> 64
    q0 = (p_lo + u0) & M
    q1 = (p_hi + u1 + (1 if q0 < p_lo else 0)) & M
    q1 = (q1 + 1) & M
    r = (u0 - q1 * DN) & M
    if r > q0:
        q1 = (q1 - 1) & M
        r = (r + DN) & M
    if r >= DN:
        q1 += 1
        r -= DN
    return q1, r


def to_int(limbs):
    return sum(v << (64 * i) for i, v in enumerate(limbs))


def divide_segments(limbs):
    """One division pass of dec_groups_kernel: (quotient limbs, remainder)."""
    m = len(limbs)
    seg = (m + W - 1) // W
    pw = [pow(B, j, D) for j in range(seg + 1)]
    A, Bm, bounds = [], [], []
    for lane in range(W):
        lo, hi = min(lane * seg, m), min(lane * seg + seg, m)
        rn = 0
        for j in range(hi - 1, lo - 1, -1):
            x = limbs[j]
            _, rn = div_2by1(rn | (x >> (64 - NORM)), (x << NORM) & M)
        A.append(pw[hi - lo])
        Bm.append(rn >> NORM)
        bounds.append((lo, hi))
    d = 1
    while d < W:  # __shfl_down_sync composition, lane l from lane l + d
        A2, B2 = A[:], Bm[:]
        for lane in range(W - d):
            B2[lane] = (A[lane] * Bm[lane + d] + Bm[lane]) % D
            A2[lane] = A[lane] * A[lane + d] % D
        A, Bm = A2, B2
        d *= 2
    q = list(limbs)
    for lane in range(W):
        lo, hi = bounds[lane]
        rn = (Bm[lane + 1] if lane + 1 < W else 0) << NORM
        for j in range(hi - 1, lo - 1, -1):
            x = limbs[j]
            q[j], rn = div_2by1(rn | (x >> (64 - NORM)), (x << NORM) & M)
    return q, Bm[0]


def put18(x):
    return "%018d" % x


def warp_addsub(x, y, nout, sub):
    """add_batch_kernel / dec_fix's warp_addsub: x + y (or x - y) mod B^nout."""
    out = list(x[:nout]) + [0] * max(0, nout - len(x))
    flip = M if sub else 0
    idle = 1 if sub else 0
    carry = idle
    for base in range(0, nout, W):
        if base >= len(y) and carry == idle:
            break
        s, g, p = [], 0, 0
        for lane in range(W):
            k = base + lane
            a = out[k] if k < nout else 0
            b = (y[k] if k < len(y) else 0) ^ flip
            t = (a + b) & M
            s.append(t)
            if t < a:
                g |= 1 << lane
            if t < a or t == M:
                p |= 1 << lane
        tt = g + p + carry
        for lane in range(W):
            k = base + lane
            if k < nout:
                out[k] = (s[lane] + ((((tt & 0xFFFFFFFF) ^ g ^ p) >> lane) & 1)) & M
        carry = tt >> 32
    return out


def rand_limbs(rng, n):
    return [rng.choice([0, M, 1, rng.randrange(B)]) for _ in range(n)]


def test_two_by_one_division():
    rng = random.Random(1)
    for t in range(20000):
        r = rng.randrange(D) if t % 3 else rng.choice([0, 1, D - 1])
        a = rng.randrange(B) if t % 5 else rng.choice([0, M, 1])
        q, rn = div_2by1((r << NORM) | (a >> (64 - NORM)), (a << NORM) & M)
        assert (q, rn >> NORM) == divmod(r * B + a, D) and rn % 16 == 0


@pytest.mark.parametrize("m", [1, 2, 5, 31, 32, 33, 63, 64, 65, 100, 479, 957])
def test_segment_scan_division(m):
    rng = random.Random(m)
    for _ in range(20):
        limbs = rand_limbs(rng, m)
        if rng.random() < 0.3:
            limbs[-1] = rng.randrange(1, 100)
        q, r = divide_segments(limbs)
        X = to_int(limbs)
        assert to_int(q) == X // D and r == X % D


def test_node_digits_by_repeated_division():
    """A node of 2^(i+1) groups: peeling the groups from the low end gives
    its zero-padded decimal string."""
    rng = random.Random(7)
    for groups in [2, 4, 8]:
        X = rng.randrange(10 ** (18 * groups))
        limbs = [(X >> (64 * i)) & M for i in range((X.bit_length() + 63) // 64 or 1)]
        digits = [""] * groups
        for g in range(groups - 1, -1, -1):
            limbs, r = divide_segments(limbs)
            digits[g] = put18(r)
        assert "".join(digits) == "%0*d" % (18 * groups, X)


@pytest.mark.parametrize("sub", [False, True])
def test_warp_sums_and_differences(sub):
    rng = random.Random(11 + sub)
    for _ in range(400):
        nx, ny = rng.randint(1, 130), rng.randint(1, 130)
        x, y = rand_limbs(rng, nx), rand_limbs(rng, ny)
        X, Y = to_int(x), to_int(y)
        if sub and X < Y:
            x, y, X, Y = y, x, Y, X
            nx, ny = ny, nx
        nout = max(nx, ny) + (0 if sub else 1)
        got = to_int(warp_addsub(x, y, nout, sub))
        assert got == ((X - Y) if sub else (X + Y)) % (B ** nout)


def test_split_correction():
    """dec_fix: while lo >= base, hi += 1 and lo -= base."""
    rng = random.Random(5)
    for _ in range(300):
        nb = rng.randint(1, 40)
        base = to_int(rand_limbs(rng, nb)) | (1 << (64 * nb - 1))
        q_true = rng.randrange(base)
        r_true = rng.randrange(base)
        short = rng.randint(0, 3)  # hi at most a few short of the quotient
        hi = max(0, q_true - short)
        lo = (q_true - hi) * base + r_true
        steps = 0
        while lo >= base:
            lo -= base
            hi += 1
            steps += 1
        assert (hi, lo) == (q_true, r_true) and steps <= 8
