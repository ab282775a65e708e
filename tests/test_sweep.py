"""The lambda scan of cmtip/autocorrelation/autocorrelation_mpi.py:99-190 on one GPU, against
the fixture made by running the unmodified reference's solve_ac_mpi rank by rank (six ranks,
every rank holding the whole image set; generations 0 and 1).

CPU: the lambdas of each rank and the kept-rank rule on the reference's own v1 / v2.
GPU: the whole sweep (shared points, kernel and right-hand side; six CG solves in one graph)
in FP64 against the reference's per-rank solutions, iteration counts and kept rank, and the
mixed-precision form's kept rank and solution."""
import numpy as np
import pytest
import torch

from conftest import rel_l2


@pytest.fixture(scope="module")
def sweep(golden):
    return golden("lambda_sweep")


def test_lambdas_match_reference_ranks(sweep):
    import cmtip_gb300.autocorrelation as acm
    M, size = int(sweep["M"]), int(sweep["size"])
    N = int(np.prod(sweep["slices"].shape))
    rl, fl = acm.sweep_lambdas(M ** 3, N, size)
    for gen in (0, 1):
        assert np.array_equal(rl, sweep[f"g{gen}_rlambdas"])
    assert np.array_equal(fl, 1e5 * 10.0 ** (np.arange(size) - size // 2))


@pytest.mark.parametrize("gen", [0, 1])
def test_selection_rule_on_reference_norms(sweep, gen):
    import cmtip_gb300.autocorrelation as acm
    keep = acm.sweep_select(gen, sweep[f"g{gen}_rlambdas"], sweep[f"g{gen}_v1"], sweep[f"g{gen}_v2"])
    assert keep == int(sweep[f"g{gen}_keep"])


def test_selection_rule_cases():
    import cmtip_gb300.autocorrelation as acm
    lam = [1.0, 2.0, 4.0, 8.0]
    # generation 0: the largest lambda among ||x|| >= mean(||x||)
    assert acm.sweep_select(0, lam, [5.0, 4.0, 1.0, 1.0], [0, 0, 0, 0]) == 1
    assert acm.sweep_select(0, lam, [1.0, 1.0, 1.0, 1.0], [9, 9, 9, 9]) == 3
    # later: the corner of the L-curve
    assert acm.sweep_select(1, lam, [5.0, 4.0, 1.0, 1.0], [0.1, 0.2, 3.5, 0.5]) == 3


@pytest.mark.gpu
@pytest.mark.parametrize("gen", [0, 1])
def test_sweep_fp64_matches_reference(sweep, gen):
    import cmtip_gb300.autocorrelation as acm
    M, size = int(sweep["M"]), int(sweep["size"])
    est = None if gen == 0 else sweep["estimate"].copy()
    ac, info = acm.solve_ac_sweep(gen, sweep["ppr"], sweep["rext"], sweep["slices"], M, orientations=sweep["quats"],
                                  ac_estimate=est, n_lambdas=size, prec=64, eps=1e-12, return_info=True,
                                  verbose=False)
    assert info["keep"] == int(sweep[f"g{gen}_keep"])
    assert np.array_equal(info["rlambdas"], sweep[f"g{gen}_rlambdas"])
    # scipy's stopping test on each rank's own system: where the residual flattens near
    # rtol ||b|| (generation 1, ~80 iterations) the reference's single-precision rounding of
    # its type-1 outputs moves the stopping iteration by a few
    its, ref_its = np.array(info["iterations"]), sweep[f"g{gen}_iterations"]
    assert np.all(np.abs(its - ref_its) <= np.maximum(1, 0.05 * ref_its)), (its, ref_its)
    errs = [rel_l2(info["solutions"][r].cpu().numpy(), sweep[f"g{gen}_solutions"][r]) for r in range(size)]
    assert max(errs) < 1e-4, errs
    assert rel_l2(info["v1"], sweep[f"g{gen}_v1"]) < 1e-5
    assert ac.dtype == np.float64 and rel_l2(ac, sweep[f"g{gen}_ac"]) < 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("gen,cg_prec", [(0, 64), (1, 64), (0, 32)])
def test_sweep_fp32_nufft_keeps_reference_rank(sweep, gen, cg_prec):
    # FP32 NUFFT with the default FP64 CG (and, in generation 0, whose flambdas stay small
    # enough for it, FP32 CG vectors)
    import cmtip_gb300.autocorrelation as acm
    M, size = int(sweep["M"]), int(sweep["size"])
    est = None if gen == 0 else sweep["estimate"].copy()
    ac, info = acm.solve_ac_sweep(gen, sweep["ppr"], sweep["rext"], sweep["slices"], M, orientations=sweep["quats"],
                                  ac_estimate=est, n_lambdas=size, prec=32, cg_prec=cg_prec, eps=1e-6,
                                  return_info=True, verbose=False)
    assert info["keep"] == int(sweep[f"g{gen}_keep"])
    assert rel_l2(ac, sweep[f"g{gen}_ac"]) < 2e-4


@pytest.mark.gpu
def test_sweep_solves_equal_single_solves(sweep):
    # the graph of six branches gives each solver exactly what its own cmt_cg_solve gives
    import cmtip_gb300.autocorrelation as acm
    M, size = int(sweep["M"]), int(sweep["size"])
    ac, info = acm.solve_ac_sweep(1, sweep["ppr"], sweep["rext"], sweep["slices"], M, orientations=sweep["quats"],
                                  ac_estimate=sweep["estimate"].copy(), n_lambdas=size, prec=64, eps=1e-12,
                                  return_info=True, verbose=False)
    ws = acm._workspace(M, 64, acm.TOEPLITZ, 1e-12, torch.device("cuda", torch.cuda.current_device()))
    solvers = ws.sweep_solvers(64, size)
    x0 = acm._support_and_x0(sweep["estimate"].copy(), M ** 3, torch.device("cuda"))[1]
    for r in (0, size - 1):
        d = solvers[r].matvec(info["solutions"][r].reshape(-1))  # any vector: only equality matters
        xs = [x0.clone()]
        acm.solve_many([solvers[r]], [d], xs, maxiter=7, rtol=0.0)
        x_one, it = solvers[r].solve(d, x0, maxiter=7, rtol=0.0)
        assert it == 7
        assert torch.equal(xs[0], x_one)
