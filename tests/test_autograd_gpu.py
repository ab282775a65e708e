"""Differentiable slicing (config 3 gradient checks): the hand-written adjoint backward
against central finite differences in FP64 and against the reference's adjoint."""
import numpy as np
import pytest
import torch

from conftest import rel_l2
from oracle import reference_port as rp

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ag():
    import cmtip_gb300.autograd as ag
    return ag


def _points(rng, n):
    return [torch.from_numpy(rng.uniform(-np.pi, np.pi, n)) for _ in range(3)]


def test_backward_vs_central_differences(ag):
    # M = 31, 200 points, FP64, step 1e-6 (config 3)
    rng = np.random.default_rng(31)
    M, N, h = 31, 200, 1e-6
    x, y, z = _points(rng, N)
    plans = ag.SlicePlans(M, prec=64, eps=1e-12).set_pts(x, y, z)
    f = torch.from_numpy(rng.standard_normal((M,) * 3)).cuda().requires_grad_(True)
    g = torch.from_numpy(rng.standard_normal(N)).cuda()
    loss = torch.dot(plans(f), g)
    loss.backward()
    grad = f.grad.detach()
    idx = rng.choice(M ** 3, 40, replace=False)
    with torch.no_grad():
        fd = []
        for k in idx:
            e = torch.zeros(M ** 3, dtype=torch.float64, device="cuda")
            e[k] = h
            e = e.reshape(f.shape)
            lp = torch.dot(plans(f + e), g)
            lm = torch.dot(plans(f - e), g)
            fd.append(float((lp - lm) / (2 * h)))
    got = grad.reshape(-1)[torch.from_numpy(idx).cuda()].cpu().numpy()
    assert rel_l2(got, np.array(fd)) < 1e-7


def test_gradcheck_small(ag):
    rng = np.random.default_rng(7)
    M, N = 7, 60
    plans = ag.SlicePlans(M, prec=64, eps=1e-12).set_pts(*_points(rng, N))
    f = torch.from_numpy(rng.standard_normal((M,) * 3)).cuda().requires_grad_(True)
    assert torch.autograd.gradcheck(lambda t: plans(t), (f,), eps=1e-6, atol=1e-8, rtol=1e-6)


def test_backward_equals_reference_adjoint(ag):
    # grad of sum_j g_j c_j is Re(sum_j g_j e^{+ik.x_j}) = M^3 * cmtip's adjoint_cpu(g) (adjoint.py:43)
    rng = np.random.default_rng(5)
    M, N = 31, 5000
    x, y, z = [rng.uniform(-np.pi, np.pi, N).astype(np.float32) for _ in range(3)]
    g = rng.standard_normal(N).astype(np.float32)
    ref = rp.adjoint_cpu(g.astype(np.complex64), x, y, z, M, use_recip_sym=True, grid_dtype=np.complex128) * M ** 3
    for prec, tol in ((64, 1e-9), (32, 1e-5)):
        plans = ag.SlicePlans(M, prec=prec, eps=1e-12 if prec == 64 else 1e-6)
        plans.set_pts(*(torch.from_numpy(a) for a in (x, y, z)))
        dt = torch.float64 if prec == 64 else torch.float32
        f = torch.zeros((M,) * 3, dtype=dt, device="cuda", requires_grad=True)
        (plans(f) * torch.from_numpy(g).cuda().to(dt)).sum().backward()
        assert rel_l2(f.grad.cpu().numpy(), ref) < tol


def test_chunked_least_squares_recomputes_slices(ag):
    from cmtip_gb300 import geometry
    rng = np.random.default_rng(9)
    M, n_img = 21, 24
    ppr, rext = geometry.ewald_detector(8)
    rext /= 0.9
    quats = geometry.random_quaternions(n_img, rng).astype(np.float32)
    data = torch.from_numpy(rng.standard_normal((n_img, ppr.shape[-1])))
    f0 = rng.standard_normal((M,) * 3)
    out = []
    for chunk in (n_img, 5):
        f = torch.from_numpy(f0).cuda().requires_grad_(True)
        loss = ag.sliced_least_squares(f, quats, ppr.reshape(3, -1), rext, data, chunk=chunk, eps=1e-12)
        loss.backward()
        out.append((float(loss.detach()), f.grad.cpu().numpy()))
    assert abs(out[0][0] - out[1][0]) <= 1e-10 * abs(out[0][0])
    assert rel_l2(out[1][1], out[0][1]) < 1e-10
    # same as slicing everything at once through Slice
    import cmtip_gb300.nufft as nf
    plans = ag.SlicePlans(M, prec=64, eps=1e-12)
    plans.set_pts_quat(nf.inverse_rotations(quats), torch.from_numpy(ppr.reshape(3, -1)), rext)
    f = torch.from_numpy(f0).cuda().requires_grad_(True)
    r = plans(f) - data.reshape(-1).cuda()
    (0.5 * torch.dot(r, r)).backward()
    assert rel_l2(f.grad.cpu().numpy(), out[0][1]) < 1e-10


def test_backward_refuses_repointed_plans(ag):
    # the adjoint plan given new points between forward and backward: the gradient would be
    # taken on the wrong points, so the backward raises instead
    rng = np.random.default_rng(33)
    M, N = 15, 300
    plans = ag.SlicePlans(M, prec=64, eps=1e-9).set_pts(*_points(rng, N))
    f = torch.from_numpy(rng.standard_normal((M,) * 3)).cuda().requires_grad_(True)
    loss = plans(f).sum()
    plans.set_pts(*_points(rng, N))
    with pytest.raises(RuntimeError, match="new points"):
        loss.backward()
