"""CPU tests of bench.py's host logic: the multi-rank path (two gloo ranks:
barrier, max-over-ranks timing, weak-scaling aggregate) and the reference arm
(the CPU port of the reference's path), which needs no GPU."""
from __future__ import annotations

import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT


def _rank(rank, world, port, out_q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ws, r, local = bench.dist_env()
    dist.barrier()
    slowest = bench.max_over_ranks(dist, 1.0 + rank, device="cpu")
    value = bench.aggregate_gcell_steps(4096 * 4096, 200 * 50, ws, slowest)
    out_q.put((r, ws, local, slowest, value))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_timing_and_weak_scaling_aggregate():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29000 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, (r, ws, local, slowest, value) in enumerate(got):
        assert (r, ws, local) == (rank, 2, rank)
        assert slowest == 2.0  # the max over ranks
        assert value == pytest.approx(4096 * 4096 * 200 * 50 * 2 / 2.0 / 1e9)


def test_reference_arm_runs_on_cpu(oracle):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--size", "256", "--steps", "3", "--warmup", "1"],
                       capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "Gcell-steps/s"
    assert line["e2e"] == {"value": line["value"], "unit": "Gcell-steps/s",
                           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["warmup"] >= 3  # at least three warm-up steps whatever is asked
