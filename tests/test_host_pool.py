"""The page-locked host pool (nn_host_alloc / nn_host_free, engine.cpp): a
buddy allocator over slabs.  Without a device its slabs are ordinary memory,
so its bookkeeping is tested here on the CPU: live blocks never overlap and
keep their contents, every block is 64-KiB aligned within its slab and at
least as large as asked, and freed blocks merge, so a computation whose
buffers double level by level (a binary-splitting tree) or repeats itself
does not make the pool grow."""
import ctypes as C
import random

import numpy as np


def lib():
    import natural_number_gb300 as nn
    L = nn.lib()
    L.nn_host_alloc.restype = C.c_void_p
    L.nn_host_alloc.argtypes = [C.c_uint64]
    L.nn_host_free.restype = None
    L.nn_host_free.argtypes = [C.c_void_p, C.c_uint64]
    L.nn_host_pool_reserved.restype = C.c_uint64
    L.nn_host_pool_reserved.argtypes = []
    return L


def fill(p, n, tag):
    a = np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_uint8)), shape=(n,))
    a[0] = tag & 255
    a[n - 1] = (tag >> 8) & 255
    a[n // 2] = (tag >> 16) & 255


def check(p, n, tag):
    a = np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_uint8)), shape=(n,))
    return (int(a[0]), int(a[n - 1]), int(a[n // 2])) == (tag & 255, (tag >> 8) & 255, (tag >> 16) & 255)


def test_blocks_disjoint_and_intact():
    L = lib()
    rng = random.Random(3)
    live = {}
    tag = 1
    for step in range(3000):
        if live and rng.random() < 0.45:
            p = rng.choice(list(live))
            n, t = live.pop(p)
            assert check(p, n, t)
            L.nn_host_free(p, n)
        else:
            n = rng.choice([16, 100, 4096, 65536, 65537, 100000, 1 << 18, 3 << 19, 1 << 21])
            p = L.nn_host_alloc(n)
            assert p and p % 16 == 0
            fill(p, n, tag)
            live[p] = (n, tag)
            tag += 1
        if step % 500 == 0:
            spans = sorted((p, p + max(n, 1 << 16)) for p, (n, _) in live.items())
            assert all(a_end <= b for (_, a_end), (b, _) in zip(spans, spans[1:]))
    for p, (n, t) in live.items():
        assert check(p, n, t)
        L.nn_host_free(p, n)


def test_doubling_levels_and_repeats_do_not_grow():
    L = lib()
    base = L.nn_host_pool_reserved()

    def tree():  # 512 blocks of 64 KiB, then 256 of 128 KiB, ... one of 32 MiB
        n, count = 1 << 16, 512
        prev = []
        while count >= 1:
            cur = [L.nn_host_alloc(n) for _ in range(count)]
            for p in prev:
                L.nn_host_free(p, n // 2)
            prev = cur
            n, count = 2 * n, count // 2
        for p in prev:
            L.nn_host_free(p, n // 2)

    tree()
    after_one = L.nn_host_pool_reserved()
    # one level live at a time (32 MiB) plus the next one: within one 64 MiB slab
    # beyond whatever the pool held before
    assert after_one - base <= 1 << 27
    for _ in range(3):
        tree()
    assert L.nn_host_pool_reserved() == after_one
