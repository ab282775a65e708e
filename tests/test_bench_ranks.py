"""The bench's multi-rank host logic on CPU (gloo, world size 2): replicas time their own
step and the line reports the slowest replica; the reference arm runs on rank 0 only."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

from conftest import REPO


def _worker(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, REPO)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        got = bench.max_over_ranks(1.5 + rank, dist, "cpu")
        # the reference arm: ranks other than 0 leave without work or output
        sys.argv = ["bench.py", "--impl", "reference", "--gpus", str(world)]
        ref = bench._run() if rank != 0 else "skipped"
        out.put((rank, got, ref))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_reference_rank_gating():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as sock:  # a free rendezvous port
        sock.bind(("127.0.0.1", 0))
        port = sock.getsockname()[1]
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert [r[1] for r in res] == [2.5, 2.5]  # both ranks see the slowest replica's time
    assert res[1][2] is None  # rank 1: no reference-arm work, no line


def test_max_over_ranks_single_process():
    sys.path.insert(0, REPO)
    import bench
    assert bench.max_over_ranks(3.25) == 3.25
