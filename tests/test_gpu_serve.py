"""The request server (continuous batching): every result equals the same
request computed alone; admission by HBM budget; oversize requests rejected."""
import time

import numpy as np
import pytest

from natural_number_gb300.synth import limbs, log_uniform_sizes

pytestmark = pytest.mark.gpu


def _norm(x):
    nz = np.flatnonzero(x)
    return x[: (int(nz[-1]) + 1) if nz.size else 1]


def _mix(n, seed, lo=3, hi=15):
    rng = np.random.default_rng(seed)
    sizes = log_uniform_sizes(seed, 2 * n, lo, hi)
    jobs = []
    for k in range(n):
        na, nb = int(sizes[2 * k]), int(sizes[2 * k + 1])
        if rng.random() < 0.2:  # division: 2n-limb dividend by an n-limb divisor
            nb = max(2, nb // 2)
            jobs.append(("div", limbs(seed * 1000 + 2 * k, 2 * nb), limbs(seed * 1000 + 2 * k + 1, nb)))
        else:
            jobs.append(("mul", limbs(seed * 1000 + 2 * k, na), limbs(seed * 1000 + 2 * k + 1, nb)))
    return jobs


def test_served_results_equal_alone_results(oracle):
    import natural_number_gb300 as nn
    jobs = _mix(120, 3)
    srv = nn.Server(0, hbm_budget=0, streams=3, div_workers=2)
    tickets = []
    for k, (kind, a, b) in enumerate(jobs):
        tickets.append(srv.submit_mul(a, b) if kind == "mul" else srv.submit_div(a, b))
        if k % 7 == 0:
            time.sleep(0.002)  # later arrivals join while earlier batches run
    results = [srv.wait(t) for t in tickets]
    stats = srv.stats()
    srv.close()
    for (kind, a, b), (res, meta) in zip(jobs, results):
        if kind == "mul":
            assert np.array_equal(res, oracle.mul(a, b))
        else:
            q, r = oracle.div(a, b)
            assert np.array_equal(_norm(res[0]), _norm(q)) and np.array_equal(_norm(res[1]), _norm(r))
        assert meta["submit"] <= meta["admit"] <= meta["done"]
    assert stats["batches"] >= 1


def test_budget_admission_and_rejection(oracle):
    import natural_number_gb300 as nn
    jobs = _mix(40, 5, 6, 13)
    srv = nn.Server(0, hbm_budget=64 << 20, streams=2, div_workers=1)
    tickets = [srv.submit_mul(a, b) if k == "mul" else srv.submit_div(a, b) for k, a, b in jobs]
    out = [srv.wait(t) for t in tickets]
    st = srv.stats()
    assert st["peak_bytes"] <= 64 << 20 or st["max_batch_jobs"] == 1
    for (kind, a, b), (res, _) in zip(jobs, out):
        if kind == "mul":
            assert np.array_equal(res, oracle.mul(a, b))
    with pytest.raises(nn.NNError) as e:
        srv.submit_mul(np.ones(1 << 22, dtype=np.uint64), np.ones(1 << 22, dtype=np.uint64))
    assert e.value.status == nn.NN_ERR_BUDGET
    srv.close()


def test_served_large_products_on_concurrent_streams():
    """Products of 2^21 limbs and more (scale 22 and up), several batches in
    flight on the server's streams at once, the twiddle tables growing while
    earlier batches run: every product equals the one computed on a plain
    context."""
    import natural_number_gb300 as nn
    sizes = [(1 << 21, 1 << 21), (300, 200), ((1 << 21) + 7, (1 << 21) - 3), (5000, 7000), ((1 << 22) - 5, 1 << 21),
             (1 << 20, (1 << 20) + 1), ((1 << 21) + 1, 4000), (1 << 21, (1 << 21) + 9)]
    pairs = [(limbs(700 + k, x), limbs(800 + k, y)) for k, (x, y) in enumerate(sizes)]
    srv = nn.Server(0, hbm_budget=0, streams=3, div_workers=1)
    ctx = nn.Context(0)
    try:
        for rnd in range(2):
            tickets = []
            for a, b in pairs:
                tickets.append(srv.submit_mul(a, b))
                time.sleep(0.001)
            for t, (a, b) in zip(tickets, pairs):
                got = srv.wait(t, 120.0)[0]
                assert np.array_equal(_norm(got), _norm(ctx.mul(a, b))), (rnd, a.size, b.size)
    finally:
        srv.close()
        ctx.close()
