"""The multi-process path of bench.py on CPU: two ranks over gloo (the GPU runs
use NCCL, one rank per GPU).  Each rank times its own replica of the workload;
the line reports the maximum over ranks, and only rank 0 runs the CPU
reference arm."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench
    r, w = bench.dist_init(world)
    bench.dist_barrier(w)
    m = bench.dist_max(10.0 * (rank + 1), w)
    args = type("A", (), {})()
    skipped = bench.run_reference(args, r, w) if r != 0 else None  # rank > 0 leaves the reference arm at once
    out.put((r, w, dist.get_backend(), m, skipped))
    bench.dist_barrier(w)
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_max(monkeypatch):
    mp = pytest.importorskip("torch.multiprocessing")
    monkeypatch.setenv("CUDA_VISIBLE_DEVICES", "")  # the ranks run on CPU (gloo) wherever the test runs
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[0] for g in got] == [0, 1] and all(g[1] == 2 and g[2] == "gloo" for g in got)
    assert all(g[3] == 20.0 for g in got)
    assert got[1][4] == 0
