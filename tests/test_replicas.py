"""The multi-rank bench path (replicas only): ranks time their own cavity and the
slowest rank's time makes the value.  Two gloo ranks on the CPU check the max
reduction and the whole-job value arithmetic; no data-path collective exists."""
import os

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = [10.0, 30.0][rank]
    total = bench.max_over_ranks(ms, dist)
    cells = 512 * 512 * 5 * world
    q.put((rank, total, cells / (total / 1e3), bench.dist_env()))
    dist.destroy_process_group()


def test_two_gloo_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29400 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, total, value, env in out:
        assert total == 30.0
        assert value == pytest.approx(512 * 512 * 5 * 2 / 0.030)
        assert env == (2, rank, 0)
