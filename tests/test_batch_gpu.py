"""Batched plans (many reconstructions, one persistent launch per NUFFT stage) and the
autotuner: a batch equals each plan executed on its own, whatever each plan's modes,
points and tuning."""
import numpy as np
import pytest
import torch

from conftest import rel_l2
from oracle import nufft as on

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nf():
    import cmtip_gb300.nufft as nf
    return nf


def _instances(rng, Ms, Ns, lim=np.pi):
    return [(M, [rng.uniform(-lim, lim, N).astype(np.float32) for _ in range(3)]) for M, N in zip(Ms, Ns)]


@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("cplx", [False, True])
def test_batched_type1_equals_single_plans(nf, prec, cplx):
    from cmtip_gb300.batch import Batch
    rng = np.random.default_rng(41)
    inst = _instances(rng, [17, 24, 9, 31], [20000, 5000, 30000, 12000])
    eps = 1e-6 if prec == 32 else 1e-7
    # bin sizes whose subgrids fit in shared memory: up to 16 cells (FP32), 8 (FP64)
    tunings = [(8, 8192), (4, 2048), (16 if prec == 32 else 2, 4096), (8, 256)]
    plans, cs = [], []
    for (M, pts), (bs, ms) in zip(inst, tunings):
        p = nf.Plan(1, M, eps=eps, isign=1, prec=prec).set_tuning(bs, ms)
        p.set_pts(*(torch.from_numpy(a) for a in pts))
        plans.append(p)
        N = pts[0].size
        cs.append(torch.from_numpy(rng.standard_normal(N) + (1j * rng.standard_normal(N) if cplx else 0)))
    b = Batch(plans)
    outs = b.execute(cs, real_out=not cplx)
    for p, c, o, (M, pts) in zip(plans, cs, outs, inst):
        single = p.execute(c, real_out=not cplx)
        assert rel_l2(o.cpu().numpy(), single.cpu().numpy()) < (1e-6 if prec == 32 else 1e-12)
        ref = on.type1(*pts, c.numpy(), M, eps=1e-13, isign=1)
        assert rel_l2(o.cpu().numpy(), ref if cplx else ref.real) < 2e-5
    # unit strengths for every plan; supports and scales per plan
    sups = [torch.from_numpy((rng.random((M,) * 3) > 0.3).astype(np.float32)) for M, _ in inst]
    outs = b.execute(None, real_out=True, support=sups, scale=[0.5, 1.0, 2.0, 3.0])
    for p, o, s, k in zip(plans, outs, sups, [0.5, 1.0, 2.0, 3.0]):
        single = p.execute(None, real_out=True, support=s, scale=k)
        assert rel_l2(o.cpu().numpy(), single.cpu().numpy()) < (1e-6 if prec == 32 else 1e-12)


@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("real_out", [False, True])
def test_batched_type2_equals_single_plans(nf, prec, real_out):
    from cmtip_gb300.batch import Batch
    rng = np.random.default_rng(42)
    inst = _instances(rng, [21, 16, 33], [15000, 40000, 8000])
    eps = 1e-6 if prec == 32 else 1e-7
    plans, fs = [], []
    for (M, pts), bs in zip(inst, (4, 8, 16 if prec == 32 else 2)):
        p = nf.Plan(2, M, eps=eps, isign=-1, prec=prec).set_tuning(bs, 4096)
        p.set_pts(*(torch.from_numpy(a) for a in pts))
        plans.append(p)
        fs.append(torch.from_numpy(rng.standard_normal((M,) * 3) + 1j * rng.standard_normal((M,) * 3)))
    b = Batch(plans)
    outs = b.execute(fs, real_out=real_out)
    for p, f, o, (M, pts) in zip(plans, fs, outs, inst):
        single = p.execute(f, real_out=real_out)
        assert rel_l2(o.cpu().numpy(), single.cpu().numpy()) < (1e-6 if prec == 32 else 1e-12)
        ref = on.type2(*pts, f.numpy(), eps=1e-13, isign=-1)
        assert rel_l2(o.cpu().numpy(), ref.real if real_out else ref) < 2e-5
    # new points on one plan are picked up by the next execute
    pts2 = [a[::-1].copy() for a in inst[1][1]]
    plans[1].set_pts(*(torch.from_numpy(a) for a in pts2))
    o = b.execute(fs, real_out=real_out)[1]
    ref = on.type2(*pts2, fs[1].numpy(), eps=1e-13, isign=-1)
    assert rel_l2(o.cpu().numpy(), ref.real if real_out else ref) < 2e-5


def test_batch_rejects_mixed_plans(nf):
    from cmtip_gb300.batch import Batch
    a = nf.Plan(1, 9, eps=1e-6)
    with pytest.raises(ValueError):
        Batch([a, nf.Plan(2, 9, eps=1e-6)])
    with pytest.raises(ValueError):
        Batch([a, nf.Plan(1, 9, eps=1e-3)])
    with pytest.raises(ValueError):
        a.set_tuning(64, 4096)


def test_autotuner_picks_a_valid_tuning(nf, tmp_path, monkeypatch):
    from cmtip_gb300 import geometry, tune
    monkeypatch.setenv("CMT_TUNE_CACHE", str(tmp_path / "tune.json"))
    rng = np.random.default_rng(3)
    ppr, rext = geometry.ewald_detector(32)
    rext /= 0.9
    quats = geometry.random_quaternions(40, rng).astype(np.float32)
    inv = nf.inverse_rotations(quats)
    pprd = torch.from_numpy(ppr.reshape(3, -1))
    data = torch.randn(40 * ppr.shape[-1], device="cuda")
    res = tune.autotune(1, 31, lambda p: p.set_pts_quat(inv, pprd, rext), data, bin_sizes=(4, 8), maxsubs=(2048, 8192))
    assert (res["bin_size"], res["maxsub"]) in {(4, 2048), (4, 8192), (8, 2048), (8, 8192)}
    assert not res["cached"] and len(res["table"]) == 4
    again = tune.autotune(1, 31, lambda p: p.set_pts_quat(inv, pprd, rext), data, bin_sizes=(4, 8),
                          maxsubs=(2048, 8192))
    assert again["cached"] and again["bin_size"] == res["bin_size"]
    # the tuned plan gives the same transform
    p = tune.apply(nf.Plan(1, 31), res).set_pts_quat(inv, pprd, rext)
    q = nf.Plan(1, 31).set_pts_quat(inv, pprd, rext)
    assert rel_l2(p.execute(data, real_out=True).cpu().numpy(), q.execute(data, real_out=True).cpu().numpy()) < 1e-6


def test_batched_reconstruction_equals_per_instance_stages(nf):
    # three reconstructions of different size through the batched stages, against the
    # single-instance entry points (compute_slices, match_orientations, solve_ac)
    from cmtip_gb300 import alignment, autocorrelation, geometry
    from cmtip_gb300.batch import BatchedReconstruction, Instance
    rng = np.random.default_rng(44)
    inst, acs = [], []
    for M, P, n_img in ((21, 16, 40), (25, 8, 60), (31, 16, 25)):
        ppr, rext = geometry.ewald_detector(P)
        rext /= 0.9
        rho = geometry.gaussian_particle(M, 40, 0.3 * M, rng)
        ac = geometry.autocorrelation_of(rho).astype(np.float32)
        q = geometry.random_quaternions(n_img, rng).astype(np.float32)
        inst.append(Instance(M, ppr.reshape(3, -1), rext, None, q))
        acs.append(ac)
    br = BatchedReconstruction(inst, eps=1e-6)
    sl = br.slices(acs)
    for x, ac, s in zip(inst, acs, sl):
        ref = alignment.compute_slices(x.orientations, x.ppr.numpy(), x.rext, torch.from_numpy(ac).cuda())
        assert rel_l2(s.cpu().numpy(), ref.cpu().numpy()) < 1e-6
        x.images = s.reshape(-1, x.n_pix)
    refs = geometry.uniform_quaternions(300)
    res = br.match(acs, 300, ref_orientations=refs)
    for x, ac, (q, info) in zip(inst, acs, res):
        q1, info1 = alignment.match_orientations(0, x.ppr.numpy().reshape(3, 1, -1), x.rext,
                                                 x.images.reshape(-1, 1, x.n_pix), torch.from_numpy(ac).cuda(), 300,
                                                 ref_orientations=refs, return_info=True)
        assert np.array_equal(info["index"], info1["index"])
    sol = br.solve(maxiter=10)
    for x, s in zip(inst, sol):
        ref = autocorrelation.solve_ac(0, x.ppr.numpy().reshape(3, 1, -1), x.rext,
                                       x.images.reshape(-1, 1, x.n_pix), x.M, orientations=x.orientations,
                                       maxiter=10, rtol=0.0, verbose=False)
        assert rel_l2(s.cpu().numpy(), ref.cpu().numpy() if torch.is_tensor(ref) else ref) < 1e-4


def test_batched_derived_plans_keep_the_extended_window(nf):
    # a batch of derived (2M) plans spreads through the extended register window like a
    # single derived plan; results equal each plan's own execute
    from cmtip_gb300.batch import Batch
    rng = np.random.default_rng(45)
    srcs, ders = [], []
    for M, N in ((17, 30000), (24, 12000), (31, 20000)):
        p = nf.Plan(1, M, eps=1e-6, isign=1).set_tuning(5, 4096)
        p.set_pts(*(torch.from_numpy(rng.uniform(-np.pi, np.pi, N).astype(np.float32)) for _ in range(3)))
        srcs.append(p)
        ders.append(p.derive(1, 2 * M, isign=1))
    outs = Batch(ders).execute(None, real_out=True, fft_order=True, scale=[1.0, 2.0, 0.5])
    for d, o, k in zip(ders, outs, [1.0, 2.0, 0.5]):
        single = d.execute(None, real_out=True, fft_order=True, scale=k)
        assert rel_l2(o.cpu().numpy(), single.cpu().numpy()) < 1e-6
