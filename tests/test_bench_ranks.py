"""The multi-process bookkeeping of bench.py (replicas, one process per GPU)
on two CPU processes with the gloo backend: every rank sees the slowest
rank's time and the whole-job rate counts the units of all ranks."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")
    rate = bench.whole_job_rate(1000, 4, world, ms)
    out.put((rank, ms, rate))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_rate_with_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [15.0, 15.0]
    # 2 ranks x 4 steps x 1000 units in 15 ms
    assert res[0][2] == pytest.approx(2 * 4 * 1000 / 0.015)


def test_single_process_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5, None, "cpu") == 12.5


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_ensemble_instances_shard_over_ranks(world):
    """Every instance lands on exactly one rank and the per-rank DOF stay
    within one instance of each other (largest first, least loaded rank)."""
    sys.path.insert(0, ROOT)
    import numpy as np
    import bench
    rng = np.random.default_rng(2026)
    sides = [int(x) for x in rng.choice([64, 128, 192, 256, 384, 512], size=64)]
    work = [n * n for n in sides]
    shards = bench.shard_instances(work, world)
    assert len(shards) == world
    assert sorted(i for s in shards for i in s) == list(range(len(work)))
    loads = [sum(work[i] for i in s) for s in shards]
    assert max(loads) - min(loads) <= max(work)
    assert bench.shard_instances([5, 1], 4)[2:] == [[], []]  # more ranks than instances: idle ranks
