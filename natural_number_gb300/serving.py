"""Served request stream: multiply/divide jobs with Poisson arrivals.

Jobs: `share_div` of them divisions of a 2n-limb dividend by an n-limb divisor,
the rest products, with sizes log-uniform in [2^lo, 2^hi] limbs; limbs are
uniform u64 (operands are slices of one SplitMix64-seeded pool, chosen so
their top limb is nonzero).  A closed-loop run (a window of outstanding
requests) measures capacity; open-loop runs submit at Poisson arrival times
at fractions of that capacity and report p50/p99 latency and limbs/s.  A
sample of results is recomputed alone (one request, nothing else on the
server) and compared bit for bit.

Throughput counts n_a + n_b limbs per product and 3n per division (dividend
plus divisor).
"""
from __future__ import annotations

import time

import numpy as np

from .synth import limbs, log_uniform_sizes, splitmix64


class ServeWorkload:
    def __init__(self, count: int, lo: float = 8, hi: float = 22, share_div: float = 0.1, seed: int = 9):
        self.pool = limbs(seed, (1 << int(np.ceil(hi))) * 2 + 64)
        sizes = log_uniform_sizes(seed + 1, 2 * count, lo, hi)
        u = (splitmix64(seed + 2, count) >> np.uint64(11)).astype(np.float64) / 2**53
        offs = (splitmix64(seed + 3, 2 * count) % np.uint64(1 << int(np.ceil(hi)))).astype(np.int64)
        self.jobs = []
        for k in range(count):
            if u[k] < share_div:
                n = max(2, int(sizes[2 * k]) // 2)
                a, b = self._slice(offs[2 * k], 2 * n), self._slice(offs[2 * k + 1], n)
                self.jobs.append(("div", a, b, 3 * n))
            else:
                na, nb = int(sizes[2 * k]), int(sizes[2 * k + 1])
                a, b = self._slice(offs[2 * k], na), self._slice(offs[2 * k + 1], nb)
                self.jobs.append(("mul", a, b, na + nb))

    def _slice(self, off: int, n: int) -> np.ndarray:
        off = int(off)
        while self.pool[off + n - 1] == 0:
            off += 1
        return self.pool[off:off + n]

    @property
    def limbs_total(self) -> int:
        return sum(j[3] for j in self.jobs)


def _submit(srv, job):
    kind, a, b, _ = job
    return srv.submit_mul(a, b) if kind == "mul" else srv.submit_div(a, b)


def closed_loop(srv, W: ServeWorkload, window: int = 64) -> dict:
    t0 = time.perf_counter()
    pending, lat = [], []
    for job in W.jobs:
        pending.append(_submit(srv, job))
        if len(pending) >= window:
            _, meta = srv.wait(pending.pop(0))
            lat.append(meta["done"] - meta["submit"])
    for t in pending:
        _, meta = srv.wait(t)
        lat.append(meta["done"] - meta["submit"])
    dt = time.perf_counter() - t0
    return {"seconds": dt, "limbs_per_s": W.limbs_total / dt, "jobs_per_s": len(W.jobs) / dt}


def open_loop(srv, W: ServeWorkload, rate: float, seed: int = 4) -> dict:
    """Submits job k at its Poisson arrival time (rate jobs/s); latency is
    completion minus arrival on the server's clock.  A second thread waits
    for the results in submission order while the submissions go on, so a
    result's buffer is released once it is read and a long stream does not
    hold every product in host memory at once."""
    import queue
    import threading

    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, len(W.jobs)))
    tickets: queue.Queue = queue.Queue()
    metas, errors = [], []

    def consume():
        while True:
            t = tickets.get()
            if t is None:
                return
            try:
                metas.append(srv.wait(t)[1])
            except Exception as e:  # reported after the stream; keep draining
                errors.append(e)

    waiter = threading.Thread(target=consume, daemon=True)
    waiter.start()
    t0 = time.perf_counter()
    try:
        for job, at in zip(W.jobs, arrivals):
            delay = at - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            tickets.put(_submit(srv, job))
    finally:
        tickets.put(None)
        waiter.join()
    if errors:
        raise errors[0]
    lat = np.array([m["done"] - m["submit"] for m in metas])
    t_first = min(m["submit"] for m in metas)
    t_last = max(m["done"] for m in metas)
    return {"rate_jobs_per_s": rate, "p50_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_ms": float(np.percentile(lat, 99) * 1e3), "mean_ms": float(lat.mean() * 1e3),
            "limbs_per_s": W.limbs_total / (t_last - t_first)}


def _norm(x: np.ndarray) -> np.ndarray:
    """Without leading zero limbs (natural::std)."""
    nz = np.flatnonzero(x)
    return x[: (int(nz[-1]) + 1) if nz.size else 1]


def check_sample(srv, ctx, W: ServeWorkload, every: int = 25) -> bool:
    """Recomputes a sample alone (on the server, nothing else queued) and on
    a plain context, and compares with a mixed-run result (as values: the
    server returns normalised quotients, natural::_div may keep a leading
    zero limb as the reference's does)."""
    ok = True
    for k in range(0, len(W.jobs), every):
        kind, a, b, _ = W.jobs[k]
        mixed_t = [_submit(srv, W.jobs[j]) for j in range(k, min(k + 8, len(W.jobs)))]
        mixed = srv.wait(mixed_t[0])[0]
        for t in mixed_t[1:]:
            srv.wait(t)
        alone = srv.wait(_submit(srv, W.jobs[k]))[0]
        direct = ctx.mul(a, b) if kind == "mul" else ctx.div(a, b)
        if kind == "mul":
            ok &= np.array_equal(mixed, alone) and np.array_equal(alone, direct)
        else:
            ok &= all(np.array_equal(_norm(x), _norm(y)) and np.array_equal(_norm(y), _norm(z))
                      for x, y, z in zip(mixed, alone, direct))
    return bool(ok)


def measure(count: int = 400, fractions=(0.5, 0.8), budget: int = 64 << 30) -> dict:
    import natural_number_gb300 as nn
    W = ServeWorkload(count)
    srv = nn.Server(0, hbm_budget=budget, streams=3, div_workers=2)
    ctx = nn.Context(0)
    _submit_warm = [srv.submit_mul(limbs(1, 4096), limbs(2, 4096)), srv.submit_div(limbs(3, 8192), limbs(4, 4096))]
    for t in _submit_warm:
        srv.wait(t)
    cap = closed_loop(srv, W)
    runs = [open_loop(srv, W, f * cap["jobs_per_s"], seed=11 + i) for i, f in enumerate(fractions)]
    exact = check_sample(srv, ctx, W)
    stats = srv.stats()
    srv.close()
    ctx.close()
    return {"workload": "%d jobs, %d%% divisions (2n by n limbs), sizes log-uniform in [2^8, 2^22] limbs, "
                        "Poisson arrivals" % (count, round(100 * sum(j[0] == 'div' for j in W.jobs) / count)),
            "hbm_budget_bytes": budget, "capacity": cap, "open_loop": runs, "bit_exact_sample": exact,
            "max_concurrent_batches": stats["max_concurrent_batches"], "batches": stats["batches"],
            "peak_admitted_bytes": stats["peak_bytes"]}
