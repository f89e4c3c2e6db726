"""The replicas path of bench.py at world size 2 on CPU (gloo): rank
discovery, whole-job throughput from the slowest rank, and the reference
arm's non-zero ranks leaving without work."""

import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist

    class A:
        pass

    r, w, local = bench.dist_init(A())
    rate, t = bench.job_throughput(3, 1.5 + rank, w)  # rank 1 is the slow one
    dist.barrier()
    dist.destroy_process_group()
    q.put((r, w, local, rate, t))


@pytest.mark.timeout(120)
def test_two_rank_replica_aggregation():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=100) for _ in ps)
    for p in ps:
        p.join(timeout=30)
    assert [o[:3] for o in out] == [(0, 2, 0), (1, 2, 1)]
    for _, _, _, rate, t in out:
        assert t == pytest.approx(2.5)             # max over ranks
        assert rate == pytest.approx(3 * 2 / 2.5)  # units of both ranks / slowest time


def _ref_worker(rank, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    class A:
        pass

    if rank == 1:
        q.put(("ret", bench.reference_arm(A())))  # leaves before any attribute of the run is read
    else:
        import torch.distributed as dist

        bench.dist_init(A())
        q.put(("rank0", None))
        dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_reference_arm_nonzero_rank_exits():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_ref_worker, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = sorted(q.get(timeout=100) for _ in ps)
    for p in ps:
        p.join(timeout=30)
    assert got == [("rank0", None), ("ret", None)]
