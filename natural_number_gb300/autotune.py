"""Autotuner for the tile/radix/batch shapes.

Sweeps, on the GPU it runs on:
  - the NTT pass split: levels of the contiguous pass ("r_last") and the most
    levels of a strided column pass ("r_col"), timed on one product per
    scale; and for batched transforms at scales 13-17 ("batch_r_last@s"),
    timed on a batch of balanced products (a batch merges small tiles, so
    its best split differs);
  - the batch shapes: persistent CTAs per SM ("batch_blocks_per_sm") and the
    shortest operand sent down the NTT route in a batch ("batch_ntt_min"),
    timed on the uneven-size workload.
Every candidate's product is checked against the first candidate's (all
choices compute the same exact product).  Writes the best values to
tuning.json beside this file; Context() applies that file at creation
(NN_TUNING=<path> picks another file, NN_TUNING=off none).

    python -m natural_number_gb300.autotune [--n-exps 14,17,20,22,24,26,27] [--batch-scales 13,14,15,16,17] [--jobs 1024]
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TUNING = os.path.join(HERE, "tuning.json")


def _time(fn, reps: int) -> float:
    import torch
    s = torch.cuda.current_stream()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    fn()
    torch.cuda.synchronize()
    a.record(s)
    for _ in range(reps):
        fn()
    b.record(s)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def tune_passes(ctx, n_exps) -> tuple[dict, dict]:
    """Per transform scale s = n_exp + 1: the pass split of one balanced
    2^n_exp x 2^n_exp product (ties keep the default split)."""
    import torch

    from .synth import limbs
    best, log = {}, {}
    for n_exp in n_exps:
        n = 1 << n_exp
        s = n_exp + 1
        a = torch.from_numpy(limbs(11, n)).cuda()
        b = torch.from_numpy(limbs(12, n)).cuda()
        out = torch.empty(2 * n, dtype=torch.uint64, device="cuda")
        ref = None
        results = {}
        reps = max(2, min(20, (1 << 26) // n))
        for r_last in (11, 9, 10, 12):
            for r_col in (9, 8, 7):
                ctx.set_tunable("r_last@%d" % s, r_last)
                ctx.set_tunable("r_col@%d" % s, r_col)
                ms = _time(lambda: ctx.mul_device(out, a, b), reps)
                if ref is None:
                    ref = out.clone()
                elif not torch.equal(ref, out):
                    raise RuntimeError(f"s={s} r_last={r_last} r_col={r_col} changed the product")
                results[f"{r_last},{r_col}"] = ms
        first = min(results.values())
        pick = next(k for k, v in results.items() if v <= first * 1.01)  # default order breaks near-ties
        r_last, r_col = map(int, pick.split(","))
        ctx.set_tunable("r_last@%d" % s, r_last)
        ctx.set_tunable("r_col@%d" % s, r_col)
        best["r_last@%d" % s] = r_last
        best["r_col@%d" % s] = r_col
        log["mul_2^%d_ms" % n_exp] = results
        del a, b, out, ref
    return best, log


def tune_batch_scales(ctx, scales) -> tuple[dict, dict]:
    """The pass split at the scales where products are usually batched
    (2^12-2^16-limb operands): timed on a batch of balanced products at each
    scale, 2^24 transform words in all (with the small-tile merging a batch
    does, the best split differs from a lone product's)."""
    import torch

    from .workloads import MulJob
    best, log = {}, {}
    for s in scales:
        n = (1 << (s - 1)) - 1
        count = max(16, (1 << 24) >> s)
        g = torch.Generator(device="cuda")
        g.manual_seed(s)
        a = torch.randint(0, 2**62, (n * count,), dtype=torch.int64, device="cuda", generator=g).view(torch.uint64)
        b = torch.randint(0, 2**62, (n * count,), dtype=torch.int64, device="cuda", generator=g).view(torch.uint64)
        out = torch.zeros(2 * n * count, dtype=torch.uint64, device="cuda")
        jobs = (MulJob * count)()
        for j in range(count):
            jobs[j] = MulJob(a.data_ptr() + 8 * n * j, n, b.data_ptr() + 8 * n * j, n, out.data_ptr() + 16 * n * j)
        sizes = np.full(count, n, dtype=np.uint64)
        results, ref = {}, None
        for r_last in (11, 10, 9, 8, 7, 6, 5):
            if r_last > s - 2:
                continue
            ctx.set_tunable("batch_r_last@%d" % s, r_last)
            plan = ctx.batch(sizes, sizes)
            ms = _time(lambda: plan.run_jobs(jobs), 5)
            ctx.synchronize()
            plan.close()
            if ref is None:
                ref = out.clone()
            elif not torch.equal(ref, out):
                raise RuntimeError(f"s={s} r_last={r_last} changed a product")
            results[str(r_last)] = ms
        first = min(results.values())
        pick = int(next(k for k, v in results.items() if v <= first * 1.01))
        ctx.set_tunable("batch_r_last@%d" % s, pick)
        best["batch_r_last@%d" % s] = pick
        log["batch_scale_%d_ms" % s] = results
        del a, b, out, ref
    return best, log


def tune_batch(ctx, jobs: int) -> tuple[dict, dict]:
    """CTAs per SM, the shortest operand sent down the NTT route, and the
    residues per pass item, on an uneven workload of `jobs` products; every
    setting must give the same products."""
    import torch

    from .workloads import UnevenProducts
    W = UnevenProducts(jobs, seed=5)
    results = {}
    ref = None
    for per_sm in (2, 3):
        for ntt_min in (64, 128, 256, 384):
            for item in (8192, 16384, 32768):
                ctx.set_tunable("batch_blocks_per_sm", per_sm)
                ctx.set_tunable("batch_ntt_min", ntt_min)
                ctx.set_tunable("batch_item_words", item)
                plan = ctx.batch(W.sa, W.sb)
                ms = _time(lambda: plan.run_jobs(W.jobs_batch), 3)
                ctx.synchronize()
                if ref is None:
                    ref = W.out_batch.clone()
                elif not torch.equal(ref, W.out_batch):
                    raise RuntimeError(f"per_sm={per_sm} ntt_min={ntt_min} item={item} changed a product")
                plan.close()
                results[f"{per_sm},{ntt_min},{item}"] = ms
    best = min(results, key=results.get)
    per_sm, ntt_min, item = map(int, best.split(","))
    ctx.set_tunable("batch_blocks_per_sm", per_sm)
    ctx.set_tunable("batch_ntt_min", ntt_min)
    ctx.set_tunable("batch_item_words", item)
    return ({"batch_blocks_per_sm": per_sm, "batch_ntt_min": ntt_min, "batch_item_words": item},
            {"batch_%d_ms" % jobs: results})


def main() -> None:
    import torch

    from . import Context
    ap = argparse.ArgumentParser()
    ap.add_argument("--n-exps", default="14,17,20,22,24,26,27")
    ap.add_argument("--batch-scales", default="13,14,15,16,17")
    ap.add_argument("--jobs", type=int, default=1024)
    ap.add_argument("--out", default=TUNING)
    args = ap.parse_args()
    os.environ["NN_TUNING"] = "off"
    ctx = Context(0)
    t0 = time.time()
    best, log = {}, {}
    b, l = tune_passes(ctx, [int(x) for x in args.n_exps.split(",")])
    best.update(b)
    log.update(l)
    b, l = tune_batch_scales(ctx, [int(x) for x in args.batch_scales.split(",")])
    best.update(b)
    log.update(l)
    b, l = tune_batch(ctx, args.jobs)
    best.update(b)
    log.update(l)
    doc = {"tunables": best, "device": torch.cuda.get_device_name(0), "seconds": round(time.time() - t0, 1),
           "timings_ms": log}
    with open(args.out, "w") as f:
        json.dump(doc, f, indent=1)
    print(json.dumps(doc))


def apply(ctx, path: str | None = None) -> dict:
    """Applies tuning.json (or NN_TUNING) to a context; returns what it set."""
    path = path or os.environ.get("NN_TUNING", TUNING)
    if path == "off" or not os.path.exists(path):
        return {}
    with open(path) as f:
        tun = json.load(f).get("tunables", {})
    for k, v in tun.items():
        ctx.set_tunable(k, int(v))
    return tun


if __name__ == "__main__":
    main()
