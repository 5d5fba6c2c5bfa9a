"""Multi-GPU form of the path: independent replicas (one grid per GPU), timed
with a barrier and the max over ranks.  The host logic is exercised here with
two gloo ranks on CPU (no GPU, no data-path collective)."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, times, out):
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mx = bench.reduce_max(times[rank], world, "cpu")
        out.put((rank, mx, bench.replica_rate(10, world, mx)))
    finally:
        dist.destroy_process_group()


def test_replica_timing_takes_max_over_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    times = [12.5, 20.0]
    procs = [ctx.Process(target=_rank, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, mx, rate in res:
        assert mx == pytest.approx(20.0)
        assert rate == pytest.approx(2 * 10 / 0.020)


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.reduce_max(3.0, 1) == 3.0
    assert bench.replica_rate(40, 1, 200.0) == pytest.approx(200.0)
