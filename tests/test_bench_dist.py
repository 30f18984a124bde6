"""The multi-rank path of bench.py on CPU: two gloo ranks, as torchrun would
start them (RANK / WORLD_SIZE / MASTER_* in the environment).  Replicas only:
the ranks share nothing but the max-over-ranks timing and the barriers."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    import sys
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(ws), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    ws_, rank_, local = bench.dist_setup()
    t = bench.dist_max(1.0 + rank, ws_)  # each rank's timing; every rank must see the max
    bench.dist_barrier(ws_)
    q.put((rank_, ws_, local, t))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_max_time():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 2, 0, 2.0), (1, 2, 1, 2.0)]


def test_single_rank_needs_no_process_group(monkeypatch):
    import bench
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert bench.dist_setup() == (1, 0, 0)
    assert bench.dist_max(3.5, 1) == 3.5
    bench.dist_barrier(1)
