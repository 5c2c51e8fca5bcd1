"""Multi-GPU is replicas only: under torchrun each rank runs an independent
replica and bench.py reduces with a barrier, the max of the per-rank times
and the sum of the per-rank work (no data-path collective).  Checked here
with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    d.barrier()
    mx = d.max(1.5 + rank)          # per-rank elapsed times
    sm = d.sum(1000.0 * (rank + 1))  # per-rank particle-steps
    d.barrier()
    q.put((rank, d.world, mx, sm))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_replicas_reduce_with_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 2, 2.5, 3000.0), (1, 2, 2.5, 3000.0)]
