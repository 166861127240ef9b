"""The bench's multi-rank path on CPU (gloo, world size 2): the ranks shard
slices with no data exchange; the only collective is the max of the step
times, and the job value counts every rank's slices."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t_step, t_warm = bench.max_over_ranks([1.0 + rank, 0.5 * (2 - rank)], world, "cpu")
    q.put((rank, t_step, t_warm, bench.job_value(world, 256, t_warm, t_step)))
    dist.destroy_process_group()


def test_two_ranks_take_the_slowest_and_count_all_slices():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    import bench
    for rank, t_step, t_warm, value in res:
        assert t_step == 2.0 and t_warm == 1.0
        assert value == pytest.approx(2 * 256 / (1.0 + bench.NOUTER * 2.0))
