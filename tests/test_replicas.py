"""The multi-GPU path is replicas only (every cell is independent): each rank
solves its own seeded grid and the job time is the slowest rank's.  Checked
here with two gloo ranks on the CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _rank(rank, world, port, out):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 100.0 + 50.0 * rank          # rank 1 is the slow one
        total = bench.max_over_ranks(ms, world)
        out[rank] = (bench.replica_seed("C3", rank), total, bench.job_rate(1000, world, 2, total))
    finally:
        dist.destroy_process_group()


def test_two_replicas_over_gloo():
    torch = pytest.importorskip("torch")
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
    (s0, t0, r0), (s1, t1, r1) = out[0], out[1]
    assert s0 != s1                                  # distinct grids per rank
    assert t0 == t1 == 150.0                         # max over ranks
    assert r0 == r1 == pytest.approx(2 * 1000 * 2 / 0.150)
