"""The multi-rank host logic of bench.py on CPU: two gloo ranks on 127.0.0.1.

Trajectories shard by index with no data-path collective: rank r, step s
runs trajectory indices (r * 1_000_003 + s) * B + i of one seed stream, so
no trajectory runs twice across ranks or steps; the only cross-rank
operations are the timing barrier and the max over ranks of the step time,
and the reported value is the whole job's trajectory-layers per second."""
import os
import socket

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, batch, steps, queue):
    import sys
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        seeds = [bench.seeds_for(rank, batch, s).tolist() for s in range(steps)]
        gathered = [None] * world
        dist.all_gather_object(gathered, seeds)
        slowest = bench.max_over_ranks(100.0 + 7.0 * rank, dist, "cpu")
        dist.barrier()
        if rank == 0:
            queue.put((gathered, slowest))
        else:
            queue.put(("rank", rank, slowest))
    finally:
        dist.destroy_process_group()


@pytest.fixture(scope="module")
def built():
    from mipt_gb300 import build
    if not os.path.exists(build.LIB):
        build.build()
    return True


def test_two_gloo_ranks_shard_trajectories_and_take_the_slowest_time(built):
    import torch.multiprocessing as mp
    import mipt_gb300 as mg
    world, batch, steps = 2, 4, 3
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, batch, steps, queue)) for r in range(world)]
    for p in procs:
        p.start()
    results = [queue.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    gathered, slowest = next(r for r in results if r[0] != "rank")
    others = [r for r in results if r[0] == "rank"]
    # The max over ranks reaches every rank.
    assert slowest == 107.0 and all(r[2] == 107.0 for r in others)
    # Each (rank, step) runs its own block of the one seed stream; no overlap.
    seen = []
    for rank, per_step in enumerate(gathered):
        for s, seeds in enumerate(per_step):
            base = (rank * 1_000_003 + s) * batch
            assert seeds == [mg.trajectory_seed(0, base + i) for i in range(batch)]
            seen.extend(seeds)
    assert len(seen) == len(set(seen)) == world * steps * batch


def test_whole_job_rate_is_weak_scaling():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    one = bench.whole_job_rate(32, 48, 1, 5, 2.0)
    assert one == 32 * 48 * 5 / 2.0
    # Same per-rank work and time on 8 ranks: 8x the whole-job rate.
    assert bench.whole_job_rate(32, 48, 8, 5, 2.0) == 8 * one
    assert bench.max_over_ranks(3.25, None, "cuda") == 3.25
