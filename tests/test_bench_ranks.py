"""bench.py's multi-rank path on CPU: world_size-2 gloo ranks (one replica per
rank, no exchange): the time taken is the slowest rank's, the value sums the
replicas, and the reference arm runs on rank 0 alone."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        slow = bench.max_over_ranks(1.5 + rank, world, device="cpu")
        q.put((rank, slow, bench.job_throughput(100, 10, slow, world)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_and_sum_the_replicas():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29000 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=5) for _ in range(2))
    assert [o[1] for o in out] == [2.5, 2.5]            # both ranks see the slower time
    assert [o[2] for o in out] == [2 * 100 * 10 / 2.5] * 2


def test_single_rank_is_the_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.0, 1) == 3.0
    assert bench.job_throughput(8, 2, 4.0, 1) == 4.0


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1"],
                       capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""
