"""The N > 1 path of bench.py: independent replicas joined only for timing
(a barrier, the maximum of the per-rank times and the sum of the units
processed), over gloo on CPU with world size 2."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    w, r, local = bench.dist_setup()
    assert (w, r, local) == (world, rank, rank)
    bench.barrier(w)
    t = bench.allmax(w, 10.0 + rank)          # per-rank "ms": the job takes the slowest
    units = bench.allsum(w, 1000.0 * (rank + 1))  # units each rank processed
    out[rank] = (t, units)
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_replicas_reduce_timings():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    assert out[0] == out[1] == (11.0, 3000.0)
