"""The multi-GPU path is replicas only: every rank renders its own frames, ranks meet at a barrier
and rank 0 reports whole-job throughput from the slowest rank's time.  This checks bench.py's
distributed helpers with two gloo ranks on the CPU (no GPU involved)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    import bench
    r, ws, local, dist = bench.dist_init()
    bench.barrier(dist)
    slowest = bench.max_over_ranks(dist, 10.0 * (rank + 1))
    out[rank] = (r, ws, local, slowest)
    dist.destroy_process_group()


def test_two_rank_replicas():
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0][:3] == (0, 2, 0) and res[1][:3] == (1, 2, 1)
    assert res[0][3] == res[1][3] == 20.0


def test_single_process_defaults(monkeypatch):
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    import bench
    assert bench.dist_init() == (0, 1, 0, None)
    assert bench.max_over_ranks(None, 3.5) == 3.5
