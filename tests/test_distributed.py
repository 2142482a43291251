"""The multi-process path of bench.py on CPU (gloo, world size 2): replicas
time independently and the job reports the slowest replica."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    try:
        mx = bench.max_over_ranks(10.0 + rank)
        dist.barrier()
        out.put((rank, mx, bench.job_rate(1000, 4, mx, world)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo():
    import torch.multiprocessing as mp
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
    assert [r[1] for r in res] == [11.0, 11.0]
    assert res[0][2] == pytest.approx(2 * 4 * 1000 / 11e-3)


def test_single_process_is_identity():
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
