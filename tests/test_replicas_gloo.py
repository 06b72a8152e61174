"""bench.py's multi-process plumbing on the CPU: two gloo ranks (the path has
no exchange step, so N GPUs run N independent replicas; ranks only agree on a
barrier, the slowest time and the summed work)."""
from __future__ import annotations

import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, results):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port),
                       "CUDA_VISIBLE_DEVICES": ""})
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import bench
    d = bench.Dist()
    d.barrier()
    results[rank] = (d.max(1.0 + rank), d.sum(10.0 * (rank + 1)), d.rank, d.world)
    d.barrier()
    d.close()


def test_two_gloo_ranks_reduce():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    port = _free_port()
    with mp.Manager() as mgr:
        results = mgr.dict()
        procs = [mp.Process(target=_worker, args=(r, 2, port, results)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=120)
        assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
        got = dict(results)
    assert got[0] == (2.0, 30.0, 0, 2)
    assert got[1] == (2.0, 30.0, 1, 2)
