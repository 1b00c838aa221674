#!/usr/bin/env python3
"""Benchmark: bit-exact 2^27 x 2^27-limb three-prime NTT multiply on GB300.

One step = one full product of two 2^27-limb operands (1 GiB each, uniform u64
limbs from SplitMix64 seeds, top limb nonzero) through the library's nn_mul:
forward transforms of both operands, pointwise product, inverse transform,
CRT + carry into 2^28 product limbs.

  value  device-resident: operands already in HBM, K steps timed with CUDA
         events on the library's stream; product limbs/s over all ranks.
  e2e    through the host-pointer API (nn_mul_host): pinned host operands
         copied in, multiplied, the product copied back, every step.
  roofline  the dominant kernel's algorithmic bytes per launch over its mean
         event-timed duration, against the measured HBM copy bandwidth.
  cpu_baseline  the oracle (CPU restatement of the reference, 1 thread) on a
         bounded sample: one 2^24 x 2^24-limb product.  The batched and
         served workloads carry their own cpu_baseline: the oracle on every
         host core, one job a process (all 4096 products; a stratified
         sample of the served stream).

Inputs (2 GiB operands, 6 GiB of residues per transform) are far larger than
the 129 MB L2, so no flush is needed between steps.  Multi-GPU runs are
independent replicas (weak scaling); `--impl reference` times the CPU path.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "NTT-mul limbs/s (bit-exact) batched vs plain on GB300; % HBM roofline; p99"
UNIT = "limbs/s"
N_EXP = 27
SEED_A, SEED_B = 1000 + (1 << N_EXP), 7777 + (1 << N_EXP)
FALLBACK_HBM_GBS = 6800.0

# Algorithmic bytes per launch of each kernel for a product of na x nb limbs
# at transform length L (three primes, 8-byte residues):
#   load+first pass reads the limbs once per prime and writes residues,
#   a strided/contiguous pass reads and writes every residue once,
#   pointwise reads two transforms and writes one, the CRT scan reads the
#   residues and writes the product limbs.
def kernel_bytes(name: str, na: int, nb: int, L: int) -> float:
    if name.startswith("ntt_fwd_load"):
        return 4.0 * (na + nb) + 24.0 * L  # mean operand length: one launch per operand
    if name.startswith("ntt_fwd_") or name.startswith("ntt_inv_"):
        return 48.0 * L
    if name in ("ntt_pointwise", "ntt_fused_row_pass"):
        return 72.0 * L  # fused: reads both transforms, writes one
    if name == "crt_carry_scan":
        return 24.0 * L + 8.0 * (na + nb)
    return 0.0


def mul_algorithmic_bytes(na: int, nb: int, L: int) -> float:
    """16(na+nb) + 192 L: two load+column passes, two row passes (one fused
    with the pointwise product and the inverse row pass), the inverse column
    pass fused with CRT and carry."""
    return 16.0 * (na + nb) + 192.0 * L


def measured_traffic(kernel: str, L: int):
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum)
    from the committed ncu summary profiles/traffic.txt, whose lines read
    `<kernel> <bytes per launch> <transform length L of the capture>`; the
    capture is taken on a smaller case and scaled by L, since a pass moves
    every residue once."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    try:
        for line in open(path):
            f = line.split()
            if len(f) >= 3 and f[0] == kernel and not line.startswith("#"):
                return float(f[1]) * L / float(f[2])
    except OSError:
        pass
    return None


def measured_instructions(kernel: str, L: int):
    """Warp instructions per launch from the committed ncu summary
    profiles/instructions.txt (`<kernel> <instructions per launch> <L of the
    capture>`), scaled by L like measured_traffic."""
    path = os.path.join(ROOT, "profiles", "instructions.txt")
    try:
        for line in open(path):
            f = line.split()
            if len(f) >= 3 and f[0] == kernel and not line.startswith("#"):
                return float(f[1]) * L / float(f[2])
    except OSError:
        pass
    return None


def peaks() -> tuple[float, str]:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=10)

    def summary(self) -> dict:
        rows = []
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9 and f[1].replace(".", "").isdigit():
                    rows.append(f)
        finally:
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        busy = [x for x in sm if x >= 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(busy), "sm_max_mhz": float(rows[0][2]), "reasons": reasons,
                "samples": len(rows), "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit())}


def measure_batched(ctx, steps: int, warmup: int, count: int = 4096) -> dict:
    """Uneven-size batch: `count` products with operand lengths drawn
    independently log-uniform in [2^6, 2^18] limbs, once one nn_mul per
    product (the unbatched path, run from a C loop) and once as one planned
    batch (persistent work-queue launch replayed from a CUDA graph); both on
    the same device-resident operands, timed with CUDA events, results compared."""
    import torch

    from natural_number_gb300.workloads import UnevenProducts
    W = UnevenProducts(count)
    stream = torch.cuda.current_stream()

    def timed(fn, reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    ctx.mul_each(W.jobs_plain)
    plain_ms = timed(lambda: ctx.mul_each(W.jobs_plain), max(2, steps // 3))
    t0 = time.perf_counter()
    plan = ctx.batch(W.sa, W.sb)
    plan_s = time.perf_counter() - t0
    for _ in range(max(warmup, 1)):
        plan.run_jobs(W.jobs_batch)
    batch_ms = timed(lambda: plan.run_jobs(W.jobs_batch), steps)
    ctx.synchronize()
    identical = bool(torch.equal(W.out_plain, W.out_batch))
    out = {"workload": "%d products, operand lengths log-uniform in [2^6, 2^18] limbs (independent), "
                       "%d product limbs in total, %.0f%% of products on the NTT route"
                       % (count, W.limbs_total, 100 * W.ntt_fraction(ctx.get_tunable("batch_ntt_min"),
                                                                      ctx.get_tunable("batch_school_balanced"))),
           "plain_ms": plain_ms, "batched_ms": batch_ms,
           "plain_limbs_per_s": W.limbs_total / (plain_ms / 1e3),
           "batched_limbs_per_s": W.limbs_total / (batch_ms / 1e3),
           "speedup": plain_ms / batch_ms, "identical": identical, "work_items": plan.items,
           "plan_seconds": plan_s}
    plan.close()
    del W
    return out


def measure_square(ctx, da, n: int, steps: int, warmup: int) -> dict:
    """The 2^n-limb square of the benchmark operand (one transform, the
    fused pass squares), device-resident, CUDA-event timed."""
    import torch
    out = torch.empty(2 * n, dtype=torch.uint64, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(max(warmup, 3)):
        ctx.sqr_device(out, da)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(stream)
    for _ in range(steps):
        ctx.sqr_device(out, da)
    b.record(stream)
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / steps
    L = 2 * n
    sqr_bytes = 24.0 * n + 96.0 * L
    peak, _ = peaks()
    del out
    return {"ms_per_step": ms, "limbs_per_s": 2 * n / (ms / 1e3), "algorithmic_bytes": sqr_bytes,
            "frac": sqr_bytes / (ms / 1e3) / 1e9 / peak}


def measure_division(ctx, reps: int = 3, cpu: bool = True) -> dict:
    """A 2^22 / 2^21-limb division through the host API, twice: natural::_div
    (the reference's Newton steps, every product on the GPU) and the division
    with every step on the GPU (nn_divmod_host); both checked by q*b + r == a
    on residues mod 2^64 -/+ 1.  Beside them the oracle on one host core
    dividing 2^19 by 2^18 limbs (a bounded sample)."""
    from natural_number_gb300.synth import limbs
    from tests.gpu_util import mod_checks
    n = 1 << 21
    a, b = limbs(41, 2 * n), limbs(43, n)
    ma, mb = mod_checks(a), mod_checks(b)

    def run(fn):
        q, r = fn(a, b)
        t0 = time.perf_counter()
        for _ in range(reps):
            q, r = fn(a, b)
        sec = (time.perf_counter() - t0) / reps
        mq, mr = mod_checks(q), mod_checks(r)
        ok = all((mq[i] * mb[i] + mr[i]) % m == ma[i] for i, m in enumerate((2**64 - 1, 2**64 + 1)))
        return {"seconds": sec, "limbs_per_s": 3 * n / sec, "identity_check": bool(ok)}

    out = {"workload": "%d-limb dividend by %d-limb divisor" % (2 * n, n),
           "natural_div": run(ctx.div), "device": run(ctx.divmod)}
    if cpu:
        from oracle import Oracle
        o = Oracle("port")
        m = 1 << 18
        ca, cb = limbs(47, 2 * m), limbs(53, m)
        t0 = time.perf_counter()
        o.div(ca, cb)
        cs = time.perf_counter() - t0
        out["cpu_baseline"] = {"seconds": cs, "limbs_per_s": 3 * m / cs, "cores": 1, "kind": "port",
                               "sample": "%d-limb dividend by %d-limb divisor" % (2 * m, m)}
    return out


def measure_series(ctx) -> dict:
    """pi and e to 10^8 digits (the reference's test.cpp recipes: pi with
    2^23 terms and a 6e6-limb square root, e with 2^24 terms), trees
    evaluated level by level with each level's products batched on the GPU;
    the digit strings are compared with the reference's SHA-256 digests.
    Each runs twice: the first call (page-locking host memory, growing the
    twiddle tables) is reported as first_call_seconds, the second as
    seconds."""
    import hashlib
    golden = json.load(open(os.path.join(ROOT, "tests", "golden", "golden.json")))
    out = {}
    for name in ("pi", "e"):
        c = golden["big_" + name][0]

        def run():
            if name == "pi":
                return ctx.pi_dec_levels(c["terms"], c["acc"], c["digits"])
            return ctx.e_dec_levels(c["terms"], c["digits"])

        t0 = time.perf_counter()
        digits, _ = run()  # first call: page-locks host memory, grows tables
        cold = time.perf_counter() - t0
        del digits
        t0 = time.perf_counter()
        digits, timing = run()
        wall = time.perf_counter() - t0
        out[name] = {"digits": c["digits"], "seconds": wall, "first_call_seconds": cold,
                     "exact": hashlib.sha256(digits.encode()).hexdigest() == c["out"]["sha256"],
                     "reference_seconds_x86_1core": c.get("ref_seconds"),
                     "phases": {k: round(v, 3) for k, v in timing.items()}}
        del digits
    return out


def cpu_baseline_port() -> dict:
    """The oracle (single-threaded CPU restatement) on one 2^24 x 2^24 product."""
    from natural_number_gb300.synth import limbs
    from oracle import Oracle
    n = 1 << 24
    o = Oracle("port")
    a, b = limbs(1, n), limbs(2, n)
    t = o.time_mul(a, b, 1)
    return {"value": 2 * n / t, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "one 2^24 x 2^24-limb product (2^27 workload scaled down 8x per operand), seconds=%.2f" % t}


def _ref_worker(args):
    n, seed = args
    from natural_number_gb300.synth import limbs
    from oracle import Oracle
    o = Oracle("port")
    a, b = limbs(seed, n), limbs(seed + 1, n)
    t0 = time.perf_counter()
    o.mul(a, b)
    return time.perf_counter() - t0


REF_N_EXP = 23

# Pooled CPU baselines of the batched and served workloads: every host core
# runs the oracle restatement (the reference's algorithm, one job at a time,
# as the reference would in one process per core); workers rebuild operands
# from their seeds instead of receiving them through pipes.
_POOL_STATE: dict = {}


def _pool_init(serve_seed: int, serve_hi: float) -> None:
    from oracle import Oracle
    _POOL_STATE["oracle"] = Oracle("port")
    if serve_seed >= 0:
        from natural_number_gb300.synth import limbs
        _POOL_STATE["pool"] = limbs(serve_seed, (1 << int(serve_hi + 0.999)) * 2 + 64)


def _pool_job(task) -> float:
    """One product (from seeds, or slices of the served pool) or one division."""
    o = _POOL_STATE["oracle"]
    kind = task[0]
    if kind == "seeded":
        from natural_number_gb300.synth import limbs
        _, sa, na, sb, nb = task
        a, b = limbs(sa, na), limbs(sb, nb)
    else:
        _, oa, na, ob, nb = task
        pool = _POOL_STATE["pool"]
        a, b = pool[oa:oa + na], pool[ob:ob + nb]
    t0 = time.perf_counter()
    if kind == "div":
        o.div(a, b)
    else:
        o.mul(a, b)
    return time.perf_counter() - t0


def _pooled(tasks, serve_seed: int = -1, serve_hi: float = 0) -> tuple[float, int]:
    import multiprocessing as mp
    from oracle import build_oracle
    build_oracle()
    cores = os.cpu_count() or 1
    with mp.get_context("spawn").Pool(cores, initializer=_pool_init, initargs=(serve_seed, serve_hi)) as pool:
        t0 = time.perf_counter()
        pool.map(_pool_job, tasks, chunksize=1)
        return time.perf_counter() - t0, cores


def cpu_baseline_batched(count: int) -> dict:
    """All `count` products of the uneven batch, spread over the host cores."""
    import numpy as np

    from natural_number_gb300.synth import log_uniform_sizes
    seed = 3  # UnevenProducts' default
    sa = np.maximum(log_uniform_sizes(seed, count, 6, 18).astype(np.int64), 1)
    sb = np.maximum(log_uniform_sizes(seed + 1, count, 6, 18).astype(np.int64), 1)
    tasks = [("seeded", seed * 1000003 + 2 * j, int(sa[j]), seed * 1000003 + 2 * j + 1, int(sb[j]))
             for j in range(count)]
    tasks.sort(key=lambda t: -(t[2] + t[4]))  # longest first: the pool's tail stays short
    dt, cores = _pooled(tasks)
    total = int((sa + sb).sum())
    return {"value": total / dt, "unit": UNIT, "cores": cores, "kind": "port", "seconds": dt,
            "sample": "all %d products, one process a core, each product alone" % count}


def cpu_baseline_serving(jobs: int, every: int = 20) -> dict:
    """A stratified sample of the served stream (every `every`-th job, in
    submission order) spread over the host cores; the whole stream takes
    minutes on the CPU."""
    from natural_number_gb300.serving import ServeWorkload
    W = ServeWorkload(jobs)
    base = W.pool.ctypes.data
    tasks, total = [], 0
    for k in range(0, len(W.jobs), every):
        kind, a, b, units = W.jobs[k]
        oa, ob = (a.ctypes.data - base) // 8, (b.ctypes.data - base) // 8
        tasks.append((kind, int(oa), int(a.size), int(ob), int(b.size)))
        total += units
    tasks.sort(key=lambda t: -(t[2] + t[4]))
    dt, cores = _pooled(tasks, serve_seed=9, serve_hi=22)
    return {"value": total / dt, "unit": UNIT, "cores": cores, "kind": "port", "seconds": dt,
            "sample": "%d of %d jobs (every %d-th, %d divisions), one process a core"
                      % (len(tasks), len(W.jobs), every, sum(t[0] == "div" for t in tasks))}


def run_reference(args) -> None:
    """CPU reference arm: the oracle restatement (the reference's x86-64
    assembly does not build on this Arm host), one independent product per
    host core, so the whole CPU is used; each step is a bounded sample."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import multiprocessing as mp
    from oracle import build_oracle
    build_oracle()
    cores = os.cpu_count() or 1
    n = 1 << REF_N_EXP
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        for w in range(args.warmup):
            pool.map(_ref_worker, [(n, 17 + 2 * i) for i in range(cores)])
        t0 = time.perf_counter()
        for s in range(args.steps):
            pool.map(_ref_worker, [(n, 17 + 2 * i) for i in range(cores)])
        dt = (time.perf_counter() - t0) / args.steps
    value = cores * 2 * n / dt
    sample = "%d independent 2^%d x 2^%d-limb products per step, one per host core" % (cores, REF_N_EXP, REF_N_EXP)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic (SplitMix64)",
            "config": {"workload": "plain multiply, sampled: %s, standing in for one 2^27 x 2^27 product" % sample},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


class Legs:
    """Progress and deadlines of the bench's legs.

    Every leg writes a timestamped start and end line to stderr.  A watchdog
    thread holds each leg to a wall-clock budget and the whole run to a total
    one.  A leg that raises is recorded under "skipped" and the run goes on;
    a leg that overruns its budget is recorded the same way, the result line
    gathered so far is printed, and the process ends, since a thread stuck in
    native code cannot be stopped from Python.  Legs that would start after
    the total budget is spent are recorded as not run."""

    def __init__(self, line: dict, total_s: float):
        import threading
        self.t0 = time.perf_counter()
        self.total_end = self.t0 + total_s
        self.line = line
        self.lock = threading.Lock()
        self.current = None
        self.printed = False
        self.core_done = False
        threading.Thread(target=self._watch, daemon=True).start()

    def log(self, msg: str) -> None:
        sys.stderr.write("[bench %7.1f s] %s\n" % (time.perf_counter() - self.t0, msg))
        sys.stderr.flush()

    def skip(self, name: str, why: str) -> None:
        with self.lock:
            self.line.setdefault("skipped", {})[name] = why
        self.log("skipped %s: %s" % (name, why))

    def run(self, name: str, budget_s: float, fn, core: bool = False):
        """fn() under the leg's budget; its result, or None if it was skipped."""
        now = time.perf_counter()
        if not core and now + budget_s > self.total_end:
            self.skip(name, "not run: the bench's total time budget would be exceeded")
            return None
        with self.lock:
            self.current = (name, now + budget_s, budget_s)
        self.log("start %s (budget %.0f s)" % (name, budget_s))
        try:
            out = fn()
        except Exception as e:  # noqa: BLE001 - a failed leg is reported in the line
            with self.lock:
                self.current = None
            if core:
                raise
            self.skip(name, "failed: %s: %s" % (type(e).__name__, str(e)[:300]))
            return None
        with self.lock:
            self.current = None
        self.log("done %s in %.1f s" % (name, time.perf_counter() - now))
        return out

    def emit(self) -> None:
        with self.lock:
            if self.printed:
                return
            self.printed = True
            text = json.dumps(self.line)
        sys.stdout.write(text + "\n")
        sys.stdout.flush()

    def _watch(self) -> None:
        while True:
            time.sleep(0.5)
            with self.lock:
                cur = self.current
            if cur is None or time.perf_counter() <= cur[1]:
                continue
            name, _, budget = cur
            self.skip(name, "timed out after its %.0f s budget; the run was ended there" % budget)
            if self.core_done:
                self.emit()
            self._exit(0 if self.core_done else 1)

    def _exit(self, code: int) -> None:
        """Runs the interpreter's exit handlers (bounded) and ends the process."""
        import atexit
        import threading
        t = threading.Thread(target=atexit._run_exitfuncs, daemon=True)
        t.start()
        t.join(10.0)
        os._exit(code)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n-exp", type=int, default=N_EXP, help="operand size 2^n limbs (27 = the benchmark workload)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the uneven-size batch measurement")
    ap.add_argument("--batch-count", type=int, default=4096, help="products in the uneven-size batch")
    ap.add_argument("--no-serve", action="store_true", help="skip the served request stream")
    ap.add_argument("--serve-jobs", type=int, default=4000)
    ap.add_argument("--serve-rates", default="0.3,0.5,0.7,0.9",
                    help="open-loop arrival rates as fractions of the measured capacity")
    ap.add_argument("--no-series", action="store_true", help="skip pi and e to 10^8 digits (a few seconds)")
    ap.add_argument("--no-div", action="store_true", help="skip the 2^22 / 2^21-limb division")
    ap.add_argument("--total-budget", type=float, default=1200.0, help="seconds for the whole run")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return

    line: dict = {"metric": METRIC, "unit": UNIT, "steps": args.steps, "warmup": args.warmup,
                  "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
                  "data": "synthetic (SplitMix64 uniform u64 limbs, top limb nonzero)"}
    legs = Legs(line, args.total_budget)

    import torch

    import natural_number_gb300 as nn
    from natural_number_gb300 import replicas
    from natural_number_gb300.synth import limbs

    R = replicas.Rank.from_env()
    world, rank, local = R.world, R.rank, R.local
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    n = 1 << args.n_exp
    L = 1 << (args.n_exp + 1)
    st: dict = {}

    def setup():
        st["ctx"] = nn.Context(local)
        seed_a, seed_b = R.seeds(SEED_A, SEED_B)
        st["a"], st["b"] = limbs(seed_a, n), limbs(seed_b, n)
        st["da"] = torch.from_numpy(st["a"]).to("cuda")
        st["db"] = torch.from_numpy(st["b"]).to("cuda")
        st["out"] = torch.empty(2 * n, dtype=torch.uint64, device="cuda")
        for _ in range(max(args.warmup, 3)):
            st["ctx"].mul_device(st["out"], st["da"], st["db"])
        torch.cuda.synchronize()

    legs.run("setup", 300, setup, core=True)
    ctx, stream = st["ctx"], torch.cuda.current_stream()
    replicas.barrier(dist)

    def multiply():
        start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = nn.launch_count()
        nn.profile_enable(True)
        with ClockSampler(local) as clk:
            torch.cuda.synchronize()
            start.record(stream)
            for _ in range(args.steps):
                ctx.mul_device(st["out"], st["da"], st["db"])
            stop.record(stream)
            torch.cuda.synchronize()
        nn.profile_enable(False)
        prof = nn.profile_report()
        launches = (nn.launch_count() - l0) / args.steps
        ms = start.elapsed_time(stop) / args.steps
        ctx.synchronize()
        ms = replicas.max_over_ranks(ms, dist, "cuda")
        replicas.barrier(dist)
        # spot-check the last product with size-independent modular identities
        from tests.gpu_util import mod_checks
        prod = st["out"].cpu().numpy()
        ma, mb, mp = mod_checks(st["a"]), mod_checks(st["b"]), mod_checks(prod)
        exact = mp[0] == ma[0] * mb[0] % (2**64 - 1) and mp[1] == ma[1] * mb[1] % (2**64 + 1)
        return ms, prof, launches, clk.summary(), bool(exact)

    ms, prof, launches, clocks, exact = legs.run("multiply", 180, multiply, core=True)
    value = replicas.aggregate_rate(2 * n, world, ms)
    peak, peak_kind = peaks()
    dname, (dcount, dms) = max(prof.items(), key=lambda kv: kv[1][1])
    d_avg = dms / dcount
    d_bytes = kernel_bytes(dname, n, n, L)
    achieved = d_bytes / (d_avg / 1e3) / 1e9
    mul_bytes = mul_algorithmic_bytes(n, n, L)
    line.update({
        "value": value, "n_gpus": world, "ms_per_step": ms,
        "config": {"workload": "plain multiply, 2^%d x 2^%d limbs (%d MiB per operand), product %d limbs"
                               % (args.n_exp, args.n_exp, n * 8 >> 20, 2 * n),
                   "l2": "inputs larger than L2 (operands %d MiB, residues %d MiB per transform); no flush"
                         % (n * 8 >> 20, 24 * L >> 20),
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "bit_exact_spot_check": exact},
        "roofline": {"bound": "hbm", "kernel": dname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": measured_traffic(dname, L), "peak_kind": peak_kind,
                     "bytes_per_launch": d_bytes, "launch_ms": d_avg, "launches_per_step": dcount / args.steps},
        "mul_roofline": {"algorithmic_bytes": mul_bytes, "achieved": mul_bytes / (ms / 1e3) / 1e9,
                         "frac": mul_bytes / (ms / 1e3) / 1e9 / peak, "peak_kind": peak_kind},
        "kernels": {k: {"launches_per_step": c / args.steps, "ms_per_step": t / args.steps}
                    for k, (c, t) in prof.items()},
        "gpu_launches": launches, "clocks": clocks})
    # The passes are bound by integer issue as much as by HBM: one warp
    # instruction per scheduler (4 per SM) per cycle at the sampled SM clock
    # is the issue peak.
    inst = measured_instructions(dname, L)
    if inst and clocks.get("sm_mhz"):
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        ipeak = 4.0 * sms * clocks["sm_mhz"] * 1e6
        iach = inst / (d_avg / 1e3)
        line["issue_roofline"] = {"bound": "int_issue", "kernel": dname, "achieved": iach, "peak": ipeak,
                                  "unit": "warp inst/s", "frac": iach / ipeak, "inst_per_launch": inst,
                                  "source": "profiles/instructions.txt (ncu on a smaller transform, scaled by L); "
                                            "peak 4 per SM per cycle"}

    def e2e():
        ha = torch.from_numpy(st["a"]).pin_memory().numpy()
        hb = torch.from_numpy(st["b"]).pin_memory().numpy()
        ho = torch.empty(2 * n, dtype=torch.uint64).pin_memory().numpy()
        for _ in range(max(2, args.warmup)):
            ctx.mul(ha, hb, out=ho)
        replicas.barrier(dist)
        step_ms = []
        t0 = time.perf_counter()
        for _ in range(args.steps):
            t1 = time.perf_counter()
            ctx.mul(ha, hb, out=ho)
            step_ms.append((time.perf_counter() - t1) * 1e3)
        e_ms = (time.perf_counter() - t0) / args.steps * 1e3
        e_ms = replicas.max_over_ranks(e_ms, dist, "cuda")
        # value: the mean over the K steps; the spread shows host-side stalls
        # (the host link and memory are shared with other jobs on the machine)
        return {"value": replicas.aggregate_rate(2 * n, world, e_ms), "unit": UNIT, "ms_per_step": e_ms,
                "h2d_bytes_per_step": 16 * n, "d2h_bytes_per_step": 16 * n,
                "api": "nn_mul_host (page-locked host operands in, product out, every step)",
                "step_ms_median": statistics.median(step_ms), "step_ms_min": min(step_ms),
                "step_ms_max": max(step_ms), "step_ms": [round(x, 1) for x in step_ms]}

    if not args.no_e2e:
        r = legs.run("e2e", 180, e2e, core=True)
        line["e2e"] = r
    if rank == 0 and not args.no_cpu:
        r = legs.run("cpu_baseline", 240, cpu_baseline_port, core=True)
        line["cpu_baseline"] = r
    legs.core_done = True

    r = legs.run("square", 120, lambda: measure_square(ctx, st["da"], n, args.steps, args.warmup))
    if r:
        line["square"] = r
    del st["db"]
    if not args.no_batch:
        r = legs.run("batched", 240, lambda: measure_batched(ctx, args.steps, args.warmup, args.batch_count))
        if r:
            line["batched"] = r
            if rank == 0 and not args.no_cpu:
                c = legs.run("cpu_baseline_batched", 240, lambda: cpu_baseline_batched(args.batch_count))
                if c:
                    r["cpu_baseline"] = c
    if rank == 0 and not args.no_serve:
        from natural_number_gb300 import serving as serving_mod
        rates = tuple(float(x) for x in args.serve_rates.split(",") if x)
        r = legs.run("serving", 420, lambda: serving_mod.measure(args.serve_jobs, rates))
        if r:
            line["serving"] = r
            if not args.no_cpu:
                c = legs.run("cpu_baseline_serving", 240, lambda: cpu_baseline_serving(args.serve_jobs))
                if c:
                    r["cpu_baseline"] = c
    if rank == 0 and not args.no_series:
        r = legs.run("series", 240, lambda: measure_series(ctx))
        if r:
            line["series"] = r
    if rank == 0 and not args.no_div:
        r = legs.run("division", 180, lambda: measure_division(ctx, cpu=not args.no_cpu))
        if r:
            line["division"] = r

    if rank == 0:
        legs.emit()

    def teardown():
        st.clear()
        ctx.close()
        torch.cuda.synchronize()

    legs.run("teardown", 60, teardown, core=True)


if __name__ == "__main__":
    main()
