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


def test_summary_states_each_error_against_its_bound():
    # the line's summary repeats every measured error beside its bound (NUFFT 1e-5 at eps 1e-6,
    # solved autocorrelation 1e-4) and says whether it was met
    sys.path.insert(0, REPO)
    import bench
    line = {"value": 1.36e-3, "extras": {
        "nufft_parity": {"type1_rel_l2_vs_fp64_plan": 2.0e-6, "type2_rel_l2_vs_fp64_oracle": 3.2e-6},
        "ac_rel_l2_mixed_vs_fp64_by_iterations": {"10": 4.3e-6, "100": 1.36e-4},
        "fp32_nufft_fp64_cg": {"ac_rel_l2_vs_fp64_100it": 1.08e-4}}}
    b = bench.summarize(line)["error_bounds"]
    assert b["nufft_type1"] == {"value": 2.0e-6, "bound": 1e-5, "met": True}
    assert b["nufft_type2"]["met"] and b["ac_mixed_10it"]["met"]
    assert not b["ac_mixed_100it"]["met"] and not b["ac_fp32_nufft_fp64_cg_100it"]["met"]
    # a line without those legs carries no bounds block
    assert "error_bounds" not in bench.summarize({"value": 1.0})
