"""The multi-rank measurement logic (unomol_gb300.replicas, used by bench.py under torchrun) with two
gloo ranks on the CPU: barriers, the maximum over ranks and the whole-job rate; and the reference arm
of bench.py, which only rank 0 runs."""
import os
import subprocess
import sys

import pytest

from conftest import ROOT


def _worker(rank, ws, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(ws), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    from unomol_gb300 import replicas
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    assert replicas.env() == (ws, rank, rank)
    replicas.barrier(ws)
    mx = replicas.max_over_ranks(1.0 + rank, ws)   # rank r "took" 1 + r seconds
    rate = replicas.job_rate(10, 2.0 + 2.0 * rank, ws)
    replicas.barrier(ws)
    dist.destroy_process_group()
    q.put((rank, mx, rate))


def test_replica_aggregation_two_gloo_ranks():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 2000)
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [2.0, 2.0]          # the slowest rank's time on every rank
    assert [o[2] for o in out] == [5.0, 5.0]          # 2 ranks x 10 steps / 4 s


def test_single_rank_is_the_plain_value():
    from unomol_gb300 import replicas
    assert replicas.max_over_ranks(3.5, 1) == 3.5
    assert replicas.job_rate(7, 2.0, 1) == 3.5


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, WORLD_SIZE="2", RANK="1", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
