"""The multi-GPU path of bench.py is replicas only: every rank runs its own
instances and the ranks exchange nothing but the timing (the slowest rank's
time, over a barrier). Checked here with world_size 2 on CPU (gloo)."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier()
    got = bench.max_over_ranks(1.5 + rank, device="cpu")
    bench.barrier()
    dist.destroy_process_group()
    q.put((rank, got))


def test_max_over_ranks_with_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == {0: 2.5, 1: 2.5}


def test_single_process_needs_no_group():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.max_over_ranks(3.25, device="cpu") == 3.25
