"""The multi-GPU (replica) bookkeeping on CPU: two gloo ranks reduce their
step times to the max, split a view list without overlap, and form the
job throughput the bench reports."""
import importlib
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

R = importlib.import_module("3dgrt_kdtree_gb300.replicas")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = [3.0, 5.5][rank]
        m = R.max_over_ranks(local_ms)
        views = list(R.partition(64, rank, world))
        gathered = [None] * world
        dist.all_gather_object(gathered, views)
        out.put((rank, m, gathered, R.job_throughput(2_073_600, world, m)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_max_and_partition():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, m, gathered, thr in res:
        assert m == 5.5
        flat = [v for part in gathered for v in part]
        assert flat == list(range(64))
        assert thr == pytest.approx(2_073_600 * 2 / 5.5e-3)


def test_single_process_and_partition_edges():
    assert R.max_over_ranks(4.25) == 4.25
    assert [len(R.partition(10, r, 3)) for r in range(3)] == [4, 3, 3]
    assert list(R.partition(2, 2, 3)) == []
    with pytest.raises(ValueError):
        R.partition(5, 3, 3)
    with pytest.raises(ValueError):
        R.job_throughput(1, 1, 0.0)
