"""The multi-GPU bench path runs independent replicas (the hot path has no
exchange step): its only cross-rank logic is the aggregation, max of the
step time and sum of the work.  Exercised here with two gloo ranks on CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = [10.0, 25.0][rank]
    units = [1e9, 3e9][rank]
    q.put((rank, bench.aggregate(ms, units, dist, "cpu")))
    dist.destroy_process_group()


def test_aggregate_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    res = dict(q.get(timeout=10) for _ in range(2))
    for r in range(2):
        ms, ups = res[r]
        assert ms == 25.0
        assert abs(ups - 4e9 / 0.025) < 1.0


def test_aggregate_single_rank():
    import bench
    assert bench.aggregate(20.0, 1e9) == (20.0, 1e9 / 0.02)
