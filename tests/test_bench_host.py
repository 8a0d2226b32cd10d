"""Host logic of bench.py's multi-rank path ("replicas only"), exercised
with world_size-2 gloo ranks on CPU: the slowest rank's time is used and
throughput sums the ranks' work."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    t = 1.0 + rank  # rank 1 is slower
    tmax = bench.max_over_ranks(t, ws)
    val = bench.aggregate_throughput(1000.0, tmax, ws)
    bench.barrier(ws)
    q.put((rank, tmax, val))
    dist.destroy_process_group()


def test_replica_aggregation_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    res = sorted(q.get(timeout=5) for _ in range(2))
    for rank, tmax, val in res:
        assert tmax == 2.0
        assert val == pytest.approx(1000.0 * 2 / 2.0)


def test_single_rank_aggregation():
    import bench

    assert bench.max_over_ranks(3.0, 1) == 3.0
    assert bench.aggregate_throughput(500.0, 2.0, 1) == 250.0
