"""The multi-rank bench path on CPU (gloo, world size 2): disjoint
configurations per rank, the max-over-ranks time and the whole-job
throughput (the benchmark's N-GPU runs use the same functions over NCCL)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        seeds = bench.shard_seeds(rank, steps=3, batch=4)
        gathered = [None] * world
        dist.all_gather_object(gathered, seeds)
        ms = bench.max_over_ranks(100.0 + 50.0 * rank, "cpu")
        value = bench.job_throughput(world, 4, 3, ms)
        q.put((rank, gathered, ms, value))
    finally:
        dist.destroy_process_group()


def test_two_rank_sharding_and_timing():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, gathered, ms, value in res:
        flat = [sorted(sum(g, [])) for g in gathered]
        assert not set(flat[0]) & set(flat[1]), "ranks share configurations"
        assert ms == 150.0  # the slower rank's time on both ranks
        assert value == pytest.approx(2 * 4 * 3 / 0.150)
