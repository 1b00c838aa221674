"""The library's multi-threaded host limb arithmetic (nn_host_add_n and
friends, used by the drop-in natural above 2^16 limbs) against Python
integers: same limbs and carries as the sequential loops, in place and with
the overlaps an in-place shift by whole limbs produces.  No GPU needed."""
import ctypes as C

import numpy as np
import pytest

from natural_number_gb300.synth import limbs

u64p = C.POINTER(C.c_uint64)


def lib():
    import natural_number_gb300 as nn
    L = nn.lib()
    for name in ("nn_host_add_n", "nn_host_sub_n"):
        getattr(L, name).restype = C.c_int
        getattr(L, name).argtypes = [C.c_uint64, u64p, u64p, u64p]
    for name in ("nn_host_shl_n", "nn_host_shr_n"):
        getattr(L, name).restype = None
        getattr(L, name).argtypes = [C.c_uint, C.c_uint64, u64p, u64p]
    L.nn_host_copy.restype = None
    L.nn_host_copy.argtypes = [u64p, u64p, C.c_uint64]
    return L


def P(x, off=0):
    return C.cast(x.ctypes.data + 8 * off, u64p)


def val(x):
    return int.from_bytes(np.ascontiguousarray(x, dtype="<u8").tobytes(), "little")


N = [1 << 16, (1 << 18) + 12345, 1 << 20]


@pytest.mark.parametrize("n", N)
def test_add_sub(n):
    L = lib()
    a, b = limbs(3 + n, n), limbs(5 + n, n)
    d = np.empty(n, dtype=np.uint64)
    c = L.nn_host_add_n(n, P(d), P(a), P(b))
    assert val(d) + (c << (64 * n)) == val(a) + val(b)
    br = L.nn_host_sub_n(n, P(d), P(a), P(b))
    assert val(d) - (br << (64 * n)) == val(a) - val(b)
    # carries rippling across every chunk: all-ones plus one
    ones = np.full(n, ~np.uint64(0), dtype=np.uint64)
    one = np.zeros(n, dtype=np.uint64)
    one[0] = 1
    x = ones.copy()
    assert L.nn_host_add_n(n, P(x), P(x), P(one)) == 1 and not x.any()
    assert L.nn_host_sub_n(n, P(x), P(x), P(one)) == 1 and np.array_equal(x, ones)


@pytest.mark.parametrize("n", N)
@pytest.mark.parametrize("cl", [1, 17, 63])
def test_shifts(n, cl):
    L = lib()
    s = limbs(7 + n + cl, n)
    d = np.zeros(n + 1, dtype=np.uint64)
    L.nn_host_shl_n(cl, n, P(s), P(d))
    assert val(d) == val(s) << cl
    x = np.concatenate([s, np.zeros(1, dtype=np.uint64)])  # in place
    L.nn_host_shl_n(cl, n, P(x), P(x))
    assert val(x) == val(s) << cl
    r = np.zeros(n, dtype=np.uint64)
    L.nn_host_shr_n(cl, n, P(s), P(r))
    assert val(r) == val(s) >> cl
    y = s.copy()
    L.nn_host_shr_n(cl, n, P(y), P(y))
    assert val(y) == val(s) >> cl
    # whole-limb offsets as natural::_shl/_shr make them in place
    k = 3
    z = np.zeros(n + k + 1, dtype=np.uint64)
    z[:n] = s
    L.nn_host_shl_n(cl, n, P(z), P(z, k))
    assert val(z[k:]) == val(s) << cl
    w = s.copy()
    L.nn_host_shr_n(cl, n - k, P(w, k), P(w))
    assert val(w[: n - k]) == val(s) >> (64 * k + cl)


def test_copy():
    L = lib()
    n = (1 << 18) + 5
    s = limbs(11, n)
    d = np.zeros(n, dtype=np.uint64)
    L.nn_host_copy(P(d), P(s), n)
    assert np.array_equal(d, s)
    x = np.concatenate([s, np.zeros(7, dtype=np.uint64)])
    L.nn_host_copy(P(x, 7), P(x), n)  # overlapping: memmove
    assert np.array_equal(x[7:], s)


def test_pool_shared_by_many_threads():
    """Several host threads use the worker pool at once, many times over
    (as the request server's scheduler, its division workers and the caller
    do): every operation still completes, with the sequential results.  An
    in-place shift is not idempotent, so a task run twice or counted in the
    wrong operation shows up as a wrong value; a lost completion shows up as
    a thread that does not finish."""
    import threading
    L = lib()
    n = 1 << 16
    errors, done = [], []

    def worker(t):
        s = limbs(100 + t, n)
        want_shl = val(s) << 13
        for it in range(150):
            x = np.concatenate([s, np.zeros(1, dtype=np.uint64)])
            L.nn_host_shl_n(13, n, P(x), P(x))
            d = np.empty(n, dtype=np.uint64)
            L.nn_host_copy(P(d), P(s), n)
            if val(x) != want_shl or not np.array_equal(d, s):
                errors.append((t, it))
                return
        done.append(t)

    ts = [threading.Thread(target=worker, args=(t,), daemon=True) for t in range(6)]
    for t in ts:
        t.start()
    for t in ts:
        t.join(120)
    assert not errors, errors
    assert sorted(done) == list(range(6)), "a pool operation did not complete"
