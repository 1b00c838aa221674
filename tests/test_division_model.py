"""The GPU division's algorithm (natural_number_gb300/csrc/divide.cpp) as a
Python model with the same steps and truncations, checked on the CPU against
Python's divmod: the reciprocal is at most one unit below floor(B^(2t)/D_t)
and never above it, the quotient estimate is within one of q (so the margin
of 2 keeps it below q), and at most three corrections run."""
import random

B = 1 << 64
BASE = 32  # limbs: the base reciprocal is exact (Knuth's algorithm D on the host)


def recip(D: int, t: int) -> int:
    """V ~ B^(2t) / D for a normalised D of t limbs (divide.cpp: recip)."""
    if t <= BASE:
        return B ** (2 * t) // D
    h = (t + 1) // 2 + 1  # one guard limb
    Xh = recip(D >> (64 * (t - h)), h)
    P = D * Xh
    top = P >> (64 * (t + h))
    assert top <= 1  # the sign limb the device scans read
    E = B ** (t + h) - P
    assert abs(E) < 1 << (64 * t + 1)  # fits its low t + 1 limbs
    if top == 0:
        return Xh * B ** (t - h) + ((Xh * E) >> (128 * h))
    return Xh * B ** (t - h) - ((Xh * -E) >> (128 * h)) - 1


def divide(A: int, D: int, stats: dict):
    na, nb = (A.bit_length() + 63) // 64, (D.bit_length() + 63) // 64
    cl = (64 - D.bit_length() % 64) % 64
    Dn, An = D << cl, A << cl
    ma = na + 1
    k = ma - nb + 1
    t = k + 1
    Dt = Dn >> (64 * (nb - t)) if t <= nb else Dn << (64 * (t - nb))
    At = An >> (64 * (nb - t)) if t <= nb else An << (64 * (t - nb))
    V = recip(Dt, t)
    floor_v = B ** (2 * t) // Dt
    assert floor_v - 1 <= V <= floor_v
    q_est = (At * V) >> (128 * t)
    q = An // Dn
    assert q - 1 <= q_est <= q + 1
    q1 = max(q_est - 2, 0)
    r = An - q1 * Dn
    steps = 0
    while r >= Dn:
        r -= Dn
        q1 += 1
        steps += 1
    stats["max_steps"] = max(stats["max_steps"], steps)
    assert steps <= 3
    return q1, r >> cl


def test_division_model_bounds():
    random.seed(7)
    stats = {"max_steps": 0}
    for trial in range(300):
        nb = random.choice([1, 2, 5, 33, 40, 70, 129, 300])
        na = nb + random.choice([0, 1, 2, 5, nb // 2, nb, nb + 3, 2 * nb])
        D = random.getrandbits(64 * nb) | (1 << (64 * nb - random.randint(1, 64)))
        A = random.getrandbits(64 * na) | (1 << (64 * na - 1))
        if trial % 9 == 0:
            D = B ** nb - 1
        if trial % 9 == 1:
            D = 1 << (64 * nb - 1)
        if trial % 9 == 2 and na > nb:
            A = D * random.getrandbits(64 * (na - nb))
        if trial % 9 == 3 and na > nb:
            A = D * random.getrandbits(64 * (na - nb)) - 1
        if A < D or A <= 0:
            continue
        q, r = divide(A, D, stats)
        assert (q, r) == divmod(A, D)
    assert stats["max_steps"] <= 3
