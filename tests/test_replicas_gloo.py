"""Multi-GPU is replicas only: independent chain sets per rank, with the
slowest rank's clock and the best score over ranks as the only
cross-rank steps.  Runs bench.py's aggregation on two gloo ranks on the
CPU (127.0.0.1 rendezvous)."""
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
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}",
                            rank=rank, world_size=world)
    try:
        times = bench.max_over_ranks(dist, [1.0 + rank, 10.0 - rank], "cpu")
        best = bench.global_best(dist, [-7.5, -3.25][rank], rank, world,
                                 "cpu")
        tie = bench.global_best(dist, -1.0, rank, world, "cpu")
        out.put((rank, times, best, tie))
    finally:
        dist.destroy_process_group()


def test_two_replicas_aggregate():
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
    for rank, times, best, tie in res:
        assert times == [2.0, 10.0]
        assert best == (-3.25, 1)
        assert tie == (-1.0, 0)


def test_single_process_passthrough():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(None, [3, 4.5], "cpu") == [3.0, 4.5]
    assert bench.global_best(None, -2.0, 0, 1, "cpu") == (-2.0, 0)


def test_each_rank_sees_only_its_gpu(monkeypatch):
    """Under torchrun each rank restricts the visible GPUs to its own (the
    library links its own CUDA runtime, so torch's device choice would not
    reach it)."""
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("CUDA_VISIBLE_DEVICES", "4,5,6,7")
    assert bench.own_gpu(2) == "6"
    assert os.environ["CUDA_VISIBLE_DEVICES"] == "6"
    monkeypatch.delenv("CUDA_VISIBLE_DEVICES")
    assert bench.own_gpu(3) == "3"
    assert os.environ["CUDA_VISIBLE_DEVICES"] == "3"
