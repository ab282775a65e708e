"""CUDA orientation matching against the reference's fixtures and the FP64 oracle.

Bar: with identical model slices and images, the argmin over references is identical to
the FP64 oracle's (sklearn-equivalent float64 distances) except where the oracle's two best
distances differ by less than one FP32 rounding (counted).  Through the full pipeline
(FP32 slices at NUFFT eps 1e-6) mismatches are allowed only where the oracle's relative
gap is below 1e-5."""
import numpy as np
import pytest
import torch

from conftest import rel_l2
from cmtip_gb300 import geometry
from oracle import nufft as on
from oracle import reference_port as rp

pytestmark = pytest.mark.gpu
MODES = ["fp64", "fp32", "bf16", "bf16x3"]


@pytest.fixture(scope="module")
def al():
    import cmtip_gb300.alignment as al
    return al


def _case(M=31, n_img=48, P=16, n_atoms=40, radius=6.0, seed=3, noise=0.05):
    rng = np.random.default_rng(seed)
    rho = geometry.gaussian_particle(M, n_atoms, radius, rng)
    ac = geometry.autocorrelation_of(rho)
    ppr, rext = geometry.ewald_detector(P)
    rext /= 0.9
    quats = geometry.random_quaternions(n_img, rng).astype(np.float32)
    H, K, L = rp.gen_nonuniform_positions(quats, ppr)
    xs = [a.astype(np.float32).ravel() / rext * np.pi for a in (H, K, L)]
    I = on.type2(*xs, ac, eps=1e-12, isign=-1).real.reshape(n_img, -1)
    I *= 1.0 + noise * rng.standard_normal(I.shape)
    return dict(ac=ac.astype(np.float32), ppr=ppr, rext=rext, quats=quats, slices=I.astype(np.float32)[:, None, :])


def test_compute_slices_fixture(al, golden):
    g = golden("alignment")
    sl = al.compute_slices(g["quats"], g["ppr"], g["rext"], g["ac"])
    assert sl.dtype == np.float32 and rel_l2(sl, g["slices_model"]) < 1e-5


def test_generate_weights_fixture(al, golden):
    g = golden("alignment")
    for order, key in ((0, "w0"), (-2, "w2"), (1, "w1")):
        assert np.allclose(al.generate_weights(g["ppr"], order), g[key], rtol=1e-12, atol=0)


@pytest.mark.parametrize("mode", MODES)
def test_reference_match_test_fixture(al, golden, mode):
    # cmtip/tests/test_align.py:44-61: true orientations spliced into 100 refs, nbatches=2
    g = golden("alignment")
    np.random.seed(5)
    q = al.match_orientations(0, g["ppr"], g["rext"], g["slices"], g["ac"], 100, nbatches=2, order=0,
                              true_orientations=g["quats"], ref_orientations=geometry.uniform_quaternions(100),
                              mode=mode)
    assert np.array_equal(q, g["matched"])


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("order,nbatches", [(0, 1), (-2, 3)])
def test_matcher_same_inputs_as_oracle(al, mode, order, nbatches):
    c = _case()
    n_ref = 600
    refs = geometry.uniform_quaternions(n_ref).astype(np.float32)
    model = rp.compute_slices(refs, c["ppr"], c["rext"], c["ac"]).reshape(n_ref, -1).astype(np.float32)
    x = c["slices"].reshape(len(c["quats"]), -1)
    w = rp.generate_weights(c["ppr"], order)
    # oracle: the reference's per-batch scaling and float64 distances on the same float32 slices
    quot = n_ref // nbatches
    dist = np.zeros((n_ref, x.shape[0]))
    for b in range(nbatches):
        m = model[b * quot:(b + 1) * quot].copy()
        m *= x.std() / m.std()
        dist[b * quot:(b + 1) * quot] = rp.calc_eudist(m * w, x * w)
    ref_idx = np.argmin(dist, axis=0)
    srt = np.sort(dist, axis=0)
    tie = (srt[1] - srt[0]) <= srt[0] * 2.0 ** -23
    mt = al.Matcher(x.shape[1], mode=mode)
    dt = torch.float64 if mode == "fp64" else torch.float32
    mt.set_data(torch.from_numpy(x).to(dt), w)
    mt.set_refs(torch.from_numpy(model).to(dt), nbatches=nbatches)
    idx, d1, d2, near, n_near = mt.run()
    idx = idx.cpu().numpy()
    bad = (idx != ref_idx) & ~tie
    assert not bad.any(), (np.nonzero(bad), n_near)
    assert np.allclose(d1.cpu().numpy(), srt[0], rtol=1e-5)


@pytest.mark.parametrize("mode", MODES)
def test_full_pipeline_vs_oracle(al, mode):
    c = _case(seed=7)
    n_ref = 500
    refs = geometry.uniform_quaternions(n_ref)
    q, info = al.match_orientations(0, c["ppr"], c["rext"], c["slices"], c["ac"], n_ref, nbatches=1,
                                    ref_orientations=refs, mode=mode, return_info=True)
    rq, ridx, dist = rp.match_orientations(c["ppr"], c["rext"], c["slices"], c["ac"], refs.astype(np.float32),
                                           nbatches=1, return_distances=True)
    srt = np.sort(dist, axis=0)
    close = (srt[1] - srt[0]) <= 1e-5 * srt[0]
    bad = (info["index"] != ridx) & ~close
    assert not bad.any()


def test_bf16_matches_fp32_form_larger(al):
    # 256 images x 4096 pixels against 3000 references: the tensor-core form picks the same
    # references as the plain FP32 form (up to FP32-rounding ties of the exact re-scoring)
    c = _case(M=41, n_img=256, P=32, n_atoms=80, radius=9.0, seed=11)
    n_ref = 3000
    refs = geometry.uniform_quaternions(n_ref)
    out = {}
    for mode in ("fp32", "bf16"):
        q, info = al.match_orientations(0, c["ppr"], c["rext"], c["slices"], c["ac"], n_ref, ref_orientations=refs,
                                        mode=mode, return_info=True)
        out[mode] = info
    a, b = out["fp32"], out["bf16"]
    diff = a["index"] != b["index"]
    tie = (a["second"] - a["best"]) <= a["best"] * 2.0 ** -22
    assert not (diff & ~tie).any()
    assert np.allclose(a["best"], b["best"], rtol=1e-6)


@pytest.mark.parametrize("mode", MODES)
def test_multi_conformation_matches_reference(al, golden, mode):
    # align.py:135-213 through the unmodified reference: two volumes, nbatches 2
    g = golden("alignment_mult")
    np.random.seed(7)
    q, conf = al.match_orientations_mult(0, g["ppr"], g["rext"], g["slices"], g["ac_mult"], 60, nbatches=2,
                                         order=0, true_orientations=g["quats"],
                                         ref_orientations=geometry.uniform_quaternions(60), mode=mode)
    assert np.array_equal(conf, g["conformations"])
    assert np.array_equal(q, g["matched"])


@pytest.mark.parametrize("mode", ["bf16", "bf16x3"])
def test_grouped_launch_equals_single_runs(al, mode):
    # one persistent tensor-core launch over matchers of different image, reference and
    # pixel counts gives each matcher exactly its own run's candidates and re-scored result
    g = torch.Generator(device="cuda").manual_seed(9)
    matchers, singles = [], []
    for n_img, n_ref, n_pix in ((300, 700, 1024), (37, 2000, 4096), (1000, 256, 640), (129, 513, 2048)):
        x = torch.rand(n_img, n_pix, device="cuda", generator=g)
        m = torch.rand(n_ref, n_pix, device="cuda", generator=g)
        w = np.random.default_rng(n_pix).uniform(0.5, 1.5, n_pix)
        w /= w.sum()
        mt = al.Matcher(n_pix, mode)
        mt.set_data(x, w)
        mt.set_refs(m, nbatches=1)
        singles.append([t.clone() if torch.is_tensor(t) else t for t in mt.run()])
        matchers.append(mt)
    grouped = al.Matcher.run_many(matchers)
    for one, many in zip(singles, grouped):
        for a, b in zip(one[:4], many[:4]):
            assert torch.equal(a, b)
        assert one[4] == many[4]


def test_matcher_stage_timing(al):
    # the stage timers report the last set_data / set_refs / distance / re-scoring
    g = torch.Generator(device="cuda").manual_seed(3)
    mt = al.Matcher(1024, "bf16")
    mt.profile(True)
    mt.set_data(torch.rand(200, 1024, device="cuda", generator=g), np.full(1024, 1.0 / 1024))
    mt.set_refs(torch.rand(600, 1024, device="cuda", generator=g))
    mt.run()
    t = mt.last_ms()
    assert set(t) == {"set_data", "set_refs", "distance", "rescore"}
    assert all(v > 0 for v in t.values())


def test_bounded_waits_time_out_and_recover(al):
    # the tensor-core kernel's producer issues no loads (cmt_match_stall_loads), so the MMA and
    # epilogue waits run out after a 20 ms limit: the run reports CMT_ERR_TIMEOUT, every role
    # unwinds, and the same matcher then runs normally with the same results as before
    import ctypes
    from cmtip_gb300 import _lib
    g = torch.Generator(device="cuda").manual_seed(4)
    mt = al.Matcher(2048, "bf16")
    mt.set_data(torch.rand(300, 2048, device="cuda", generator=g), np.full(2048, 1.0 / 2048))
    mt.set_refs(torch.rand(700, 2048, device="cuda", generator=g))
    before = [t.clone() for t in mt.run()[:3]]
    lib = _lib.load()
    mt.set_wait_limit(0.02)
    _lib.check(lib.cmt_match_stall_loads(mt._h, 1))
    with pytest.raises(_lib.CmtError) as e:
        mt.run()
    assert e.value.code == _lib.CMT_ERR_TIMEOUT
    _lib.check(lib.cmt_match_stall_loads(mt._h, 0))
    mt.set_wait_limit(2.0)
    after = mt.run()[:3]
    for a, b in zip(before, after):
        assert torch.equal(a, b)
    # the context is usable by other work as well
    x = torch.ones(1000, device="cuda")
    assert float(x.sum()) == 1000.0
    with pytest.raises(ValueError):
        mt.set_wait_limit(0.0)


@pytest.mark.parametrize("mode", ["bf16", "bf16x3"])
def test_tiles_give_the_same_result(al, mode, tmp_path, monkeypatch):
    # every tile of the tensor-core kernel (references per tile, ring stages) gives the same
    # candidates and re-scored result; the autotuner leaves a valid tile set
    from cmtip_gb300 import tune
    monkeypatch.setenv("CMT_TUNE_CACHE", str(tmp_path / "tune.json"))
    g = torch.Generator(device="cuda").manual_seed(6)
    mt = al.Matcher(1536, mode)
    mt.set_data(torch.rand(400, 1536, device="cuda", generator=g), np.full(1536, 1.0 / 1536))
    mt.set_refs(torch.rand(900, 1536, device="cuda", generator=g))
    ref = [t.clone() if torch.is_tensor(t) else t for t in mt.run()]
    for bn, st in tune.TILES:
        mt.set_tile(bn, st)
        got = mt.run()
        for a, b in zip(ref[:4], got[:4]):
            assert torch.equal(a, b), (bn, st)
    res = tune.autotune_match([mt])
    assert (res["bn"], res["stages"]) in tune.TILES and len(res["table"]) == len(tune.TILES)
    assert tune.autotune_match([mt])["cached"]
    with pytest.raises(ValueError):
        mt.set_tile(64, 4)
