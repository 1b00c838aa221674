"""Batched products (one persistent launch over a work queue) against the
oracle: mixed sizes on both sides of the schoolbook/NTT switch, squares,
repeated runs of one plan (CUDA-graph replay) with new operands."""
import numpy as np
import pytest

from gpu_util import empty_dev, normalize, to_dev, to_host
from natural_number_gb300.synth import limbs, log_uniform_sizes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import natural_number_gb300 as nn
    c = nn.Context(0)
    yield c
    c.close()


def run_batch(ctx, a_list, b_list, square=None, plan=None):
    import torch
    da = [to_dev(a) for a in a_list]
    db = [da[k] if (square is not None and square[k]) else to_dev(b) for k, b in enumerate(b_list)]
    outs = [empty_dev(a.size + b.size) for a, b in zip(a_list, b_list)]
    if plan is None:
        plan = ctx.batch([a.size for a in a_list], [b.size for b in b_list], square)
    plan.run(list(zip(da, db)), outs)
    ctx.synchronize()
    torch.cuda.synchronize()
    return [to_host(o) for o in outs], plan


def test_batch_mixed_sizes_vs_oracle(ctx, oracle):
    n = 160
    sa = log_uniform_sizes(11, n, 1, 14)
    sb = log_uniform_sizes(12, n, 1, 14)
    a_list = [limbs(100 + k, int(x)) for k, x in enumerate(sa)]
    b_list = [limbs(900 + k, int(x)) for k, x in enumerate(sb)]
    outs, plan = run_batch(ctx, a_list, b_list)
    for k in range(n):
        assert np.array_equal(normalize(outs[k]), oracle.mul(a_list[k], b_list[k])), (k, sa[k], sb[k])
    assert plan.items > n


def test_batch_replay_with_new_operands(ctx, oracle):
    sizes = [(64, 64), (383, 4000), (384, 384), (5000, 3000), (20000, 20001), (1, 7), (70000, 1000)]
    a1 = [limbs(k + 1, x) for k, (x, _) in enumerate(sizes)]
    b1 = [limbs(k + 50, y) for k, (_, y) in enumerate(sizes)]
    outs, plan = run_batch(ctx, a1, b1)
    for k in range(len(sizes)):
        assert np.array_equal(normalize(outs[k]), oracle.mul(a1[k], b1[k]))
    a2 = [np.full(x, 2**64 - 1, dtype=np.uint64) for x, _ in sizes]
    b2 = [limbs(k + 500, y) for k, (_, y) in enumerate(sizes)]
    for _ in range(2):
        outs, _ = run_batch(ctx, a2, b2, plan=plan)
        for k in range(len(sizes)):
            assert np.array_equal(normalize(outs[k]), normalize(oracle.mul(a2[k], b2[k])))


def test_batch_squares_and_threshold_tunable(ctx, oracle):
    sizes = [300, 384, 1000, 4096, 9000]
    a_list = [limbs(k + 7, x) for k, x in enumerate(sizes)]
    outs, _ = run_batch(ctx, a_list, a_list, square=[1] * len(sizes))
    for k, a in enumerate(a_list):
        assert np.array_equal(normalize(outs[k]), oracle.sqr(a))
    old = {k: ctx.get_tunable(k) for k in ("batch_ntt_min", "batch_school_balanced")}
    try:
        ctx.set_tunable("batch_ntt_min", 64)  # push mid sizes onto the NTT route
        ctx.set_tunable("batch_school_balanced", 0)
        a_list = [limbs(k + 70, x) for k, x in enumerate([64, 100, 200, 383])]
        b_list = [limbs(k + 80, x) for k, x in enumerate([70, 100, 250, 383])]
        outs, _ = run_batch(ctx, a_list, b_list)
        for k in range(4):
            assert np.array_equal(normalize(outs[k]), oracle.mul(a_list[k], b_list[k]))
    finally:
        for k, v in old.items():
            ctx.set_tunable(k, v)


def test_batch_fused_last_pass_matches_unfused(ctx, oracle):
    """The fused step (second operand's last forward pass + pointwise + first
    inverse pass) and the separate steps give the same products, for two- and
    three-pass transforms, products and squares."""
    sizes = [(384, 384), (1000, 3000), (4096, 4096), (20000, 20001), (70000, 1000), (200000, 300000),
             (1200000, 1100000), (5000, 5000), (300000, 300000)]
    square = [0] * 7 + [1, 1]
    a_list = [limbs(k + 301, x) for k, (x, _) in enumerate(sizes)]
    b_list = [a_list[k] if square[k] else limbs(k + 401, y) for k, (_, y) in enumerate(sizes)]
    old = ctx.get_tunable("batch_fused")
    try:
        ctx.set_tunable("batch_fused", 0)
        plain, p0 = run_batch(ctx, a_list, b_list, square=square)
        ctx.set_tunable("batch_fused", 1)
        fused, p1 = run_batch(ctx, a_list, b_list, square=square)
    finally:
        ctx.set_tunable("batch_fused", old)
    assert p1.items < p0.items  # the pointwise and first inverse items are gone
    for k in range(len(sizes)):
        assert np.array_equal(fused[k], plain[k]), k
        want = oracle.sqr(a_list[k]) if square[k] else oracle.mul(a_list[k], b_list[k])
        assert np.array_equal(normalize(fused[k]), want), k


def test_batch_merged_tiles_match_unmerged(ctx, oracle):
    """Widened strided tiles and merged contiguous tiles (transforms of scale
    13-18, where the passes' own tiles hold 32-1024 words) give the same
    products as tile-by-tile work, and the oracle's."""
    sizes = [(2000, 2100), (3000, 3000), (6000, 5000), (10000, 12000), (30000, 30000), (60000, 60000),
             (100000, 100000), (65536, 500), (20000, 20000), (4000, 4000)]
    square = [0] * 8 + [1, 1]
    a_list = [limbs(k + 501, x) for k, (x, _) in enumerate(sizes)]
    b_list = [a_list[k] if square[k] else limbs(k + 601, y) for k, (_, y) in enumerate(sizes)]
    old = ctx.get_tunable("batch_merge")
    old_rl = {s: ctx.get_tunable("batch_r_last@%d" % s) for s in (13, 16)}
    try:
        ctx.set_tunable("batch_merge", 0)
        plain, _ = run_batch(ctx, a_list, b_list, square=square)
        ctx.set_tunable("batch_merge", 1)
        merged, _ = run_batch(ctx, a_list, b_list, square=square)
        ctx.set_tunable("batch_r_last@13", 6)  # a 6-level strided pass widened to 32 columns
        ctx.set_tunable("batch_r_last@16", 7)
        merged2, _ = run_batch(ctx, a_list, b_list, square=square)
    finally:
        ctx.set_tunable("batch_merge", old)
        for s, v in old_rl.items():
            ctx.set_tunable("batch_r_last@%d" % s, v)
    for k in range(len(sizes)):
        want = oracle.sqr(a_list[k]) if square[k] else oracle.mul(a_list[k], b_list[k])
        assert np.array_equal(normalize(plain[k]), want), k
        assert np.array_equal(merged[k], plain[k]), k
        assert np.array_equal(merged2[k], plain[k]), k


def test_batch_split_unbalanced_products(ctx, oracle):
    """Unbalanced products split into pieces of the longer operand sharing
    the shorter operand's transform (either operand the longer one), mixed
    with balanced products, squares and schoolbook jobs: the same products as
    unsplit, and the oracle's."""
    sizes = [(262144, 200), (200, 262144), (100000, 3000), (3000, 100000), (65536, 8000), (5000, 128),
             (300000, 129), (20000, 20000), (4096, 4096), (1000, 50), (150000, 20000), (2048, 2048)]
    square = [0] * 10 + [0, 1]
    a_list = [limbs(k + 701, x) for k, (x, _) in enumerate(sizes)]
    b_list = [a_list[k] if square[k] else limbs(k + 801, y) for k, (_, y) in enumerate(sizes)]
    old = ctx.get_tunable("batch_split")
    try:
        ctx.set_tunable("batch_split", 0)
        whole, p0 = run_batch(ctx, a_list, b_list, square=square)
        ctx.set_tunable("batch_split", 1)
        split, p1 = run_batch(ctx, a_list, b_list, square=square)
        split2, _ = run_batch(ctx, a_list, b_list, square=square, plan=p1)  # graph replay
    finally:
        ctx.set_tunable("batch_split", old)
    assert p1.items != p0.items
    for k in range(len(sizes)):
        want = oracle.sqr(a_list[k]) if square[k] else oracle.mul(a_list[k], b_list[k])
        assert np.array_equal(normalize(whole[k]), want), k
        assert np.array_equal(split[k], whole[k]), k
        assert np.array_equal(split2[k], whole[k]), k


def test_batch_tiny_transforms_with_largest_items(ctx, oracle):
    """Every product on the NTT route, down to transforms of 4 words, with the
    largest item size: an item's tile count is capped at its 16-bit field."""
    sizes = [(1, 1), (2, 3), (5, 5), (9, 7), (33, 31), (130, 2), (1000, 1000)]
    a_list = [limbs(k + 901, x) for k, (x, _) in enumerate(sizes)]
    b_list = [limbs(k + 951, y) for k, (_, y) in enumerate(sizes)]
    old = {k: ctx.get_tunable(k) for k in ("batch_ntt_min", "batch_item_words", "batch_school_balanced")}
    try:
        ctx.set_tunable("batch_ntt_min", 1)
        ctx.set_tunable("batch_school_balanced", 0)
        ctx.set_tunable("batch_item_words", 1 << 20)
        outs, _ = run_batch(ctx, a_list, b_list)
    finally:
        for k, v in old.items():
            ctx.set_tunable(k, v)
    for k in range(len(sizes)):
        assert np.array_equal(normalize(outs[k]), oracle.mul(a_list[k], b_list[k])), k


def test_batch_large_products_run_alone(ctx, oracle):
    """Products at the batch_solo_scale tunable's scale (22: n_a + n_b - 1 >
    2^21) run one at a time beside the batch kernel's items; the results equal
    those of the batch kernel (batch_solo_scale 0) and, for the small ones and
    a 2^20-limb square, the oracle's.  A plan of large products only launches
    no batch kernel."""
    sizes = [(1 << 21, 1 << 21), (300, 200), ((1 << 21) + 5, 1000), (5000, 7000), (1 << 20, 1 << 20),
             ((1 << 20) + 1, (1 << 20) + 1)]
    square = [0, 0, 0, 0, 1, 0]
    a_list = [limbs(k + 31, x) for k, (x, _) in enumerate(sizes)]
    b_list = [a if square[k] else limbs(k + 61, y) for k, ((_, y), a) in enumerate(zip(sizes, a_list))]
    assert ctx.get_tunable("batch_solo_scale") == 22
    outs, plan = run_batch(ctx, a_list, b_list, square=square)
    old = ctx.get_tunable("batch_solo_scale")
    try:
        ctx.set_tunable("batch_solo_scale", 0)
        ref, plan0 = run_batch(ctx, a_list, b_list, square=square)
    finally:
        ctx.set_tunable("batch_solo_scale", old)
    assert plan.items < plan0.items
    for k in range(len(sizes)):
        assert np.array_equal(outs[k], ref[k]), k
    for k in (1, 3):
        assert np.array_equal(normalize(outs[k]), oracle.mul(a_list[k], b_list[k]))
    assert np.array_equal(normalize(outs[4]), oracle.sqr(a_list[4]))
    big = [0, 2, 5]
    outs2, plan2 = run_batch(ctx, [a_list[k] for k in big], [b_list[k] for k in big])
    assert plan2.items == 0
    for j, k in enumerate(big):
        assert np.array_equal(outs2[j], outs[k])
    outs3, _ = run_batch(ctx, [a_list[k] for k in big], [b_list[k] for k in big], plan=plan2)  # replayed
    for j, k in enumerate(big):
        assert np.array_equal(outs3[j], outs[k])


def test_batch_base_case_items_vs_oracle(ctx, oracle):
    """Every product on the base-case route (batch_ntt_min above all sizes):
    single-tile and multi-tile column scans (up to 7000 positions, so tiles
    whose sums start kScanE positions before them), one-limb operands,
    all-ones limbs (the largest column sums) and squares, against the oracle."""
    sizes = [(1, 1), (1, 7), (2, 2), (33, 1), (100, 80), (383, 383), (1000, 1048), (1025, 1024), (3000, 2000),
             (5000, 2000), (2047, 1), (1, 2049)]
    a_list = [limbs(k + 301, x) for k, (x, _) in enumerate(sizes)]
    b_list = [limbs(k + 401, y) for k, (_, y) in enumerate(sizes)]
    a_list.append(np.full(1500, 2**64 - 1, dtype=np.uint64))
    b_list.append(np.full(1400, 2**64 - 1, dtype=np.uint64))
    old = ctx.get_tunable("batch_ntt_min")
    try:
        ctx.set_tunable("batch_ntt_min", 1 << 20)
        outs, _ = run_batch(ctx, a_list, b_list)
        for k in range(len(a_list)):
            assert np.array_equal(normalize(outs[k]), normalize(oracle.mul(a_list[k], b_list[k]))), k
        sq = [limbs(k + 501, x) for k, x in enumerate([1, 5, 700, 2500])]
        outs, _ = run_batch(ctx, sq, sq, square=[1] * len(sq))
        for k, a in enumerate(sq):
            assert np.array_equal(normalize(outs[k]), normalize(oracle.sqr(a))), k
    finally:
        ctx.set_tunable("batch_ntt_min", old)
