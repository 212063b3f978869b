"""bench.py's replica aggregation for N > 1 (one LP per rank per step, no
data-path collective): the whole-job time is the slowest rank's and the LP
count sums the ranks'.  Run as two gloo ranks on the CPU."""
import importlib.util
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        b = _bench()
        # rank r took (r + 1) seconds of device time and 10 (r + 1) of wall
        n, dev, wall = b.replica_totals(dist, float(rank + 1), 10.0 * (rank + 1), 3)
        out[rank] = (n, dev, wall)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_replica_totals_two_gloo_ranks():
    world = 2
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        n, dev, wall = res[rank]
        assert n == 3 * world
        assert dev == 2.0 and wall == 20.0


def test_replica_totals_single_process():
    b = _bench()
    assert b.replica_totals(None, 1.5, 2.5, 3) == (3, 1.5, 2.5)
