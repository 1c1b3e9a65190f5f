"""CPU test of the bench's multi-rank arithmetic (replicas under torchrun):
two gloo ranks on 127.0.0.1 reduce their times to the slowest one, and the
job's time per product counts every rank's products."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ws, r, local = bench.dist_env()
        slowest = bench.ranks_max(dist, 10.0 + 5.0 * rank, "cpu")  # rank 1 is the slower replica
        out.put((r, ws, local, slowest, bench.job_ms_per_product(slowest, 4, ws)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1] and all(r[1] == 2 and r[2] == r[0] for r in res)
    # both ranks see the slower replica's 15 ms; 4 products per rank, 8 in all
    assert all(r[3] == 15.0 and r[4] == 15.0 / 8 for r in res)


def test_single_rank_is_unchanged():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.ranks_max(None, 3.5, "cpu") == 3.5
    assert bench.job_ms_per_product(20.0, 20, 1) == 1.0
