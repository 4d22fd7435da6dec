"""The N > 1 host logic of bench.py on CPU: one process per rank over gloo
(127.0.0.1), every rank's timings reduced to the slowest rank's, as the GPU runs
do over NCCL (replicas: no data-path collective)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as tdist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier(tdist)
        vals = bench.max_over_ranks([1.0 + rank, 10.0 - rank, 0.5 * rank], tdist, device="cpu")
        out.put((rank, vals))
    finally:
        tdist.destroy_process_group()


def test_max_over_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    world, port = 2, _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(world):
        assert res[r] == [2.0, 10.0, 0.5]


def test_max_over_ranks_single_process():
    import bench
    assert bench.max_over_ranks([3.0, 4.5], None) == [3.0, 4.5]
