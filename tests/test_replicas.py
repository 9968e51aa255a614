"""bench.py's multi-process path on CPU: two gloo ranks, as torchrun launches
them.  The tree does not shard (every rank holds a replica), so the only
cross-rank step is the timing aggregation: the slowest rank's step time and
the units of all ranks over it."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rank 1 is the slow one in the step time, rank 0 in the e2e time
    ms, e2e = (2.0, 9.0) if rank == 0 else (5.0, 3.0)
    out = bench.aggregate_replicas(ms, e2e, 100_000, world)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, out))


def test_two_rank_aggregation():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        ms, e2e, value, e2e_value = res[r]
        assert ms == 5.0 and e2e == 9.0
        assert value == pytest.approx(2 * 100_000 / 5e-3)
        assert e2e_value == pytest.approx(2 * 100_000 / 9e-3)


def test_single_rank_passthrough():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.aggregate_replicas(4.0, 8.0, 1000, 1) == (4.0, 8.0, 1000 / 4e-3, 1000 / 8e-3)
