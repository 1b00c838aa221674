"""Multi-rank path of the benchmark on CPU: two gloo ranks run independent
replicas (their own operands, no data exchange), the elapsed time is the max
over ranks, and the whole-job rate counts both ranks' units.  The product of
each replica comes from the oracle here (no GPU in this test) and is checked
against Python integers."""
import json
import os
import socket
import subprocess
import sys
import time

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    from natural_number_gb300 import replicas
    from natural_number_gb300.synth import limbs
    from oracle import Oracle, to_int
    R = replicas.Rank.from_env()
    dist.init_process_group("gloo", rank=R.rank, world_size=R.world)
    sa, sb = R.seeds(11, 23)
    a, b = limbs(sa, 600), limbs(sb, 500)
    o = Oracle("port")
    replicas.barrier(dist)
    t0 = time.perf_counter()
    p = o.mul(a, b)
    time.sleep(0.05 * (R.rank + 1))  # rank 1 is the slow one
    ms = (time.perf_counter() - t0) * 1e3
    slowest = replicas.max_over_ranks(ms, dist, "cpu")
    replicas.barrier(dist)
    res = {"rank": R.rank, "ms": ms, "slowest": slowest, "exact": to_int(p) == to_int(a) * to_int(b),
           "a0": int(a[0]), "rate": replicas.aggregate_rate(a.size + b.size, R.world, slowest)}
    with open(os.path.join(out_dir, "rank%d.json" % R.rank), "w") as f:
        json.dump(res, f)
    dist.destroy_process_group()


def test_two_gloo_replicas(tmp_path, oracle):
    world, port = 2, _free_port()
    mp.start_processes(_rank_main, args=(world, port, str(tmp_path)), nprocs=world, join=True, start_method="spawn")
    r = [json.load(open(tmp_path / ("rank%d.json" % k))) for k in range(world)]
    assert all(x["exact"] for x in r)
    assert r[0]["a0"] != r[1]["a0"]  # each rank has its own operands
    slowest = max(x["ms"] for x in r)
    assert r[0]["slowest"] == r[1]["slowest"] == pytest.approx(slowest)
    assert r[1]["ms"] > r[0]["ms"]
    assert r[0]["rate"] == pytest.approx(world * 1100 / (slowest / 1e3))


def test_reference_arm_only_on_rank0():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert p.returncode == 0 and p.stdout.strip() == ""


def test_single_rank_identity():
    from natural_number_gb300 import replicas
    assert replicas.max_over_ranks(3.5, None) == 3.5
    assert replicas.Rank().seeds(5, 9) == (5, 9)
    assert replicas.aggregate_rate(100, 1, 1000.0) == pytest.approx(100.0)
