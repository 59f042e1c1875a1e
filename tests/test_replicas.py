"""Multi-GPU is replicas only: each rank renders the same workload on its own
GPU and bench.py combines the ranks' numbers on the host (slowest rank's
time, all ranks' rays).  This checks that combination with two gloo ranks on
the CPU; the rendering itself needs one GPU per rank."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as td  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    td.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    # rank r: device ms 100 + 10 r, e2e s 1 + r, rays 1000 (r + 1), e2e rays 900 (r + 1)
    out = bench.reduce_over_ranks(td, 100.0 + 10 * rank, 1.0 + rank, 1000 * (rank + 1), 900 * (rank + 1), "cpu")
    q.put((rank, out))
    td.destroy_process_group()


def test_reduce_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        assert got[r] == (110.0, 2.0, 3000.0, 2700.0)
