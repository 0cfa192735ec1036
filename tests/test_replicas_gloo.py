"""Replica aggregation of bench.py under torch.distributed (world size 2,
gloo on CPU, rendezvous on 127.0.0.1): the job time is the slowest rank's
and the units are summed over ranks."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms, units = bench.reduce_over_ranks(10.0 + 5.0 * rank, 1000.0 * (rank + 1), device="cpu")
    q.put((rank, ms, units))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_time_is_max_and_units_are_summed():
    torch = pytest.importorskip("torch")
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    for rank, ms, units in out:
        assert ms == 15.0 and units == 3000.0


def test_single_process_reduction_is_identity():
    pytest.importorskip("torch")
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_over_ranks(7.5, 42, device="cpu") == (7.5, 42.0)
