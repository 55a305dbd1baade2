"""bench.py's multi-rank plumbing on CPU: two gloo ranks, barrier, max over ranks and the
whole-job aggregation (replicas: no data-path collective)."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    d = bench.Dist()
    assert d.world == world and d.rank == rank
    d.barrier()
    slow = d.max(100.0 + 50.0 * rank)  # rank 1 is the slowest
    value, ms = bench.aggregate([slow], 10, d.world)
    out[rank] = (slow, value, ms)
    d.close()


def test_two_gloo_ranks_take_the_slowest():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == out[1]
    slow, value, ms = out[0]
    assert slow == 150.0
    assert value == pytest.approx(2 * 10 / 0.150)
    assert ms == pytest.approx(15.0)


def test_single_process_defaults():
    import bench
    args = bench.parse_args([])
    assert args.gpus == 1 and args.warmup >= 3 and args.steps > 0
    value, ms = bench.aggregate([1000.0], 20, 1)
    assert value == pytest.approx(20.0) and ms == pytest.approx(50.0)
