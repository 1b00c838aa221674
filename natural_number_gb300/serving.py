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


def closed_loop(srv, W: ServeWorkload, window: int = 64, wait_s: float = 30.0) -> dict:
    t0 = time.perf_counter()
    pending = []
    for job in W.jobs:
        pending.append(_submit(srv, job))
        if len(pending) >= window:
            srv.wait(pending.pop(0), wait_s)
    for t in pending:
        srv.wait(t, wait_s)
    dt = time.perf_counter() - t0
    return {"seconds": dt, "limbs_per_s": W.limbs_total / dt, "jobs_per_s": len(W.jobs) / dt}


def open_loop(srv, W: ServeWorkload, rate: float, seed: int = 4, wait_s: float = 30.0) -> dict:
    """Submits job k at its Poisson arrival time (rate jobs/s); latency is
    completion minus arrival on the server's clock.  A second thread waits
    for the results in submission order while the submissions go on, so a
    result's buffer is released once it is read and a long stream does not
    hold every product in host memory at once.  The first failed or
    overdue result (no result within `wait_s` seconds of the wait's start)
    stops the stream: submissions end and the error is raised."""
    import queue
    import threading

    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, len(W.jobs)))
    tickets: queue.Queue = queue.Queue()
    metas, errors = [], []
    failed = threading.Event()

    def consume():
        while True:
            t = tickets.get()
            if t is None:
                return
            try:
                metas.append(srv.wait(t, wait_s)[1])
            except Exception as e:  # noqa: BLE001 - raised by the submitting thread
                errors.append(e)
                failed.set()
                return

    waiter = threading.Thread(target=consume, daemon=True)
    waiter.start()
    t0 = time.perf_counter()
    try:
        for job, at in zip(W.jobs, arrivals):
            if failed.is_set():
                break
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
    return {"rate_jobs_per_s": rate, "jobs": len(metas), "p50_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_ms": float(np.percentile(lat, 99) * 1e3), "mean_ms": float(lat.mean() * 1e3),
            "max_ms": float(lat.max() * 1e3), "limbs_per_s": W.limbs_total / (t_last - t_first),
            "seconds": t_last - t_first}


def _norm(x: np.ndarray) -> np.ndarray:
    """Without leading zero limbs (natural::std)."""
    nz = np.flatnonzero(x)
    return x[: (int(nz[-1]) + 1) if nz.size else 1]


def check_sample(srv, ctx, W: ServeWorkload, every: int = 25, wait_s: float = 30.0) -> bool:
    """Recomputes a sample alone (on the server, nothing else queued) and on
    a plain context, and compares with a mixed-run result (as values: the
    server returns normalised quotients, natural::_div may keep a leading
    zero limb as the reference's does)."""
    ok = True
    for k in range(0, len(W.jobs), every):
        kind, a, b, _ = W.jobs[k]
        mixed_t = [_submit(srv, W.jobs[j]) for j in range(k, min(k + 8, len(W.jobs)))]
        mixed = srv.wait(mixed_t[0], wait_s)[0]
        for t in mixed_t[1:]:
            srv.wait(t, wait_s)
        alone = srv.wait(_submit(srv, W.jobs[k]), wait_s)[0]
        direct = ctx.mul(a, b) if kind == "mul" else ctx.div(a, b)
        if kind == "mul":
            ok &= np.array_equal(mixed, alone) and np.array_equal(alone, direct)
        else:
            ok &= all(np.array_equal(_norm(x), _norm(y)) and np.array_equal(_norm(y), _norm(z))
                      for x, y, z in zip(mixed, alone, direct))
    return bool(ok)


def measure(count: int = 400, fractions=(0.5, 0.8), budget: int = 64 << 30, check_every: int = 0,
            wait_s: float = 30.0) -> dict:
    """Capacity (closed loop), then one open-loop stream per arrival rate
    (`fractions` of capacity), then a bit-exact sample of about 200 jobs
    (every `check_every`-th job; 0 picks the spacing)."""
    import natural_number_gb300 as nn
    W = ServeWorkload(count)
    srv = nn.Server(0, hbm_budget=budget, streams=3, div_workers=2)
    ctx = nn.Context(0)
    try:
        warm = [srv.submit_mul(limbs(1, 4096), limbs(2, 4096)), srv.submit_div(limbs(3, 8192), limbs(4, 4096))]
        for t in warm:
            srv.wait(t, wait_s)
        cap = closed_loop(srv, W, wait_s=wait_s)
        runs = [open_loop(srv, W, f * cap["jobs_per_s"], seed=11 + i, wait_s=wait_s) for i, f in enumerate(fractions)]
        for f, r in zip(fractions, runs):
            r["fraction_of_capacity"] = f
        every = check_every or max(1, count // 200)
        exact = check_sample(srv, ctx, W, every=every, wait_s=wait_s)
        stats = srv.stats()
    finally:
        srv.close()
        ctx.close()
    n_div = sum(j[0] == "div" for j in W.jobs)
    return {"workload": "%d jobs, %d%% divisions (2n by n limbs), sizes log-uniform in [2^8, 2^22] limbs, "
                        "Poisson arrivals at %s of capacity" % (count, round(100 * n_div / count),
                                                                ", ".join("%g" % f for f in fractions)),
            "jobs": count, "rates": list(fractions), "hbm_budget_bytes": budget, "capacity": cap,
            "open_loop": runs, "bit_exact_sample": exact, "sample_jobs": len(range(0, count, every)),
            "max_concurrent_batches": stats["max_concurrent_batches"], "batches": stats["batches"],
            "peak_admitted_bytes": stats["peak_bytes"]}


def main() -> None:
    """python -m natural_number_gb300.serving --jobs 100000 --rates 0.3,0.5,0.7,0.9
    prints one JSON object with the capacity, each rate's p50/p99 and limbs/s,
    and the bit-exact sample's verdict."""
    import argparse
    import json
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=100000)
    ap.add_argument("--rates", default="0.3,0.5,0.7,0.9")
    ap.add_argument("--budget-gib", type=int, default=64)
    args = ap.parse_args()
    rates = tuple(float(x) for x in args.rates.split(",") if x)
    print(json.dumps(measure(args.jobs, rates, args.budget_gib << 30)), flush=True)


if __name__ == "__main__":
    main()
