"""The MTIP generation loop (cmtip/reconstruct.py:29-96, run_mtip) through this package,
against the fixture made by running the unmodified reference's run_mtip (not aligned: random
generation-0 orientations, then matching against 5000 references at the 9 A limit; short
phasing schedules, tests/golden/make_golden.py loop_fixture) with the same seeds.

The hand-offs are what the test pins: generation 0's solve from the stub generator's
orientations, the phased autocorrelation as the next estimate (and its support), the
orientations matched on the clipped images, and the support and density carried from one
phasing to the next."""
import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _run(L, **kw):
    from cmtip_gb300 import reconstruct
    data = {"pixel_position_reciprocal": L["ppr"], "reciprocal_extent": float(L["rext"]),
            "intensities": L["slices"], "orientations": L["quats_true"]}
    got = {}

    def keep(g, ck):
        got[g] = {k: (v.detach().cpu().numpy().copy() if torch.is_tensor(v) else np.array(v, copy=True))
                  for k, v in ck.items() if k in ("orientations", "ac", "ac_phased", "support_", "rho_")
                  and v is not None}

    np.random.seed(int(L["np_seed"]))
    reconstruct.run_mtip(data, int(L["M"]), aligned=False, n_iterations=int(L["generations"]),
                         rng=np.random.default_rng(int(L["stub_seed"])), phase_iterations=int(L["phase_n_iterations"]),
                         nER=int(L["phase_nER"]), nHIO=int(L["phase_nHIO"]), on_generation=keep, verbose=False, **kw)
    return got


def test_mtip_loop_fp64_matches_reference(golden):
    L = golden("mtip_loop")
    got = _run(L, prec=64, match_mode="fp64", phase_prec=64, eps=1e-12)
    assert sorted(got) == list(range(int(L["generations"])))
    for g in got:
        if g > 0:
            # the same matched reference for every image
            assert np.array_equal(got[g]["orientations"], L[f"g{g}_orientations"]), g
            assert rel_l2(got[g]["ac"], L[f"g{g}_ac"]) < 1e-4, g
        assert np.array_equal(got[g]["support_"], L[f"g{g}_support_"]), g
        assert rel_l2(got[g]["rho_"], L[f"g{g}_rho_"]) < 1e-4, g
        assert rel_l2(got[g]["ac_phased"], L[f"g{g}_ac_phased"]) < 1e-4, g


def test_mtip_loop_default_forms_run(golden):
    # the fast forms (mixed-precision solve, BF16 matching, FP32 phasing) through the same
    # loop: every generation's hand-off is produced and finite
    L = golden("mtip_loop")
    got = _run(L)
    for g in got:
        assert np.all(np.isfinite(got[g]["ac_phased"]))
        assert got[g]["support_"].dtype == np.bool_ and got[g]["support_"].any()
        if g > 0:
            assert got[g]["orientations"].shape == (L["slices"].shape[0], 4)


def test_mtip_loop_writes_and_resumes_checkpoints(golden, tmp_path):
    from cmtip_gb300 import reconstruct
    L = golden("mtip_loop")
    data = {"pixel_position_reciprocal": L["ppr"], "reciprocal_extent": float(L["rext"]),
            "intensities": L["slices"], "orientations": L["quats_true"]}
    kw = dict(aligned=True, phase_iterations=1, nER=3, nHIO=3, verbose=False, prec=64, phase_prec=64, eps=1e-12)
    np.random.seed(3)
    reconstruct.run_mtip(data, int(L["M"]), output=str(tmp_path), n_iterations=2, **kw)
    ck = reconstruct.load_checkpoint(str(tmp_path / "checkpoint_g1.npz"))
    assert ck["generation"] == 1 and ck["support_"].dtype == np.bool_
    # resuming from generation 1 runs generation 2 only, from the saved phasing state
    seen = []
    reconstruct.run_mtip(data, int(L["M"]), n_iterations=3, checkpoint=ck, on_generation=lambda g, c: seen.append(g),
                         **kw)
    assert seen == [2]
