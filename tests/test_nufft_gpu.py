"""CUDA NUFFT (through the C ABI) against the FP64 oracle and the reference's fixtures.

Tolerances: FP32 plans at requested eps 1e-6 must reach relative L2 <= 1e-5 against the
FP64 oracle; FP64 plans at eps 1e-12 reach <= 1e-10."""
import numpy as np
import pytest
import torch

from conftest import rel_l2
from oracle import nufft as on
from oracle import reference_port as rp

pytestmark = pytest.mark.gpu

TOL32 = 1e-5
TOL64 = 1e-10


@pytest.fixture(scope="module")
def nf():
    import cmtip_gb300.nufft as nf
    return nf


def _pts(rng, N, lim=np.pi):
    return [rng.uniform(-lim, lim, N).astype(np.float32) for _ in range(3)]


def _uniform_points(M):
    ls = np.linspace(-1, 1, M + 1)
    ls = (ls[:-1] + ls[1:]) / 2
    h, k, l = np.meshgrid(ls, ls, ls, indexing="ij")
    return [(np.pi * a.ravel()).astype(np.float32) for a in (h, k, l)]


def test_forward_uniform_known_answer(nf):
    # restates cmtip/tests/test_nufft.py:40-49 with a synthetic AC
    from cmtip_gb300 import geometry
    rng = np.random.default_rng(3)
    rho = geometry.gaussian_particle(25, 30, 5.0, rng)
    ac = geometry.autocorrelation_of(rho).astype(np.float32)
    H, K, L = _uniform_points(25)
    calc = nf.forward_gpu(ac.copy(), H, K, L, support=None, use_recip_sym=True).real
    calc_np = np.fft.fftshift(np.fft.fftn(np.fft.ifftshift(ac)).real)
    assert np.mean(np.abs(calc_np.ravel() - calc)) < 1e-4 * max(1.0, np.abs(calc_np).mean())


def test_adjoint_uniform_known_answer(nf):
    # restates cmtip/tests/test_nufft.py:71-79
    from cmtip_gb300 import geometry
    rng = np.random.default_rng(4)
    M = 17
    rho = geometry.gaussian_particle(M, 10, 3.0, rng)
    ivol = np.fft.fftshift(np.abs(np.fft.fftn(np.fft.ifftshift(rho))) ** 2).astype(np.float32)
    H, K, L = _uniform_points(M)
    ac_np = np.fft.fftshift(np.fft.ifftn(np.fft.ifftshift(ivol)).real)
    calc = nf.adjoint_gpu(ivol.ravel(), H, K, L, M)
    assert np.mean(np.abs(ac_np - calc)) < 1e-4 * max(1.0, np.abs(ac_np).mean())


@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("M", [15, 16])
@pytest.mark.parametrize("isign", [-1, 1])
def test_type1_vs_oracle(nf, prec, M, isign):
    rng = np.random.default_rng(M + isign + prec)
    N = 20000
    x, y, z = _pts(rng, N, lim=2.9 * np.pi)
    eps, tol = (1e-6, TOL32) if prec == 32 else (1e-12, TOL64)
    c = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    ref = on.type1(x, y, z, c, M, eps=1e-13, isign=isign)
    p = nf.Plan(1, M, eps=eps, isign=isign, prec=prec).set_pts(torch.from_numpy(x), torch.from_numpy(y),
                                                               torch.from_numpy(z))
    got = p.execute(torch.from_numpy(c)).cpu().numpy()
    assert rel_l2(got, ref) < tol
    # real strengths through the R2C path, real-part output, FFT mode order
    cr = rng.standard_normal(N)
    ref = on.type1(x, y, z, cr, M, eps=1e-13, isign=isign)
    got = p.execute(torch.from_numpy(cr)).cpu().numpy()
    assert rel_l2(got, ref) < tol
    got = p.execute(torch.from_numpy(cr), real_out=True, fft_order=True).cpu().numpy()
    assert rel_l2(got, np.fft.ifftshift(ref.real)) < tol


@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("M", [15, 16])
@pytest.mark.parametrize("isign", [-1, 1])
def test_type2_vs_oracle(nf, prec, M, isign):
    rng = np.random.default_rng(100 + M + isign + prec)
    N = 20000
    x, y, z = _pts(rng, N, lim=2.9 * np.pi)
    eps, tol = (1e-6, TOL32) if prec == 32 else (1e-12, TOL64)
    f = rng.standard_normal((M,) * 3) + 1j * rng.standard_normal((M,) * 3)
    ref = on.type2(x, y, z, f, eps=1e-13, isign=isign)
    p = nf.Plan(2, M, eps=eps, isign=isign, prec=prec).set_pts(torch.from_numpy(x), torch.from_numpy(y),
                                                               torch.from_numpy(z))
    assert rel_l2(p.execute(torch.from_numpy(f)).cpu().numpy(), ref) < tol
    # real-part output through the Hermitian C2R path
    assert rel_l2(p.execute(torch.from_numpy(f), real_out=True).cpu().numpy(), ref.real) < tol
    fr = rng.standard_normal((M,) * 3)
    ref = on.type2(x, y, z, fr, eps=1e-13, isign=isign)
    assert rel_l2(p.execute(torch.from_numpy(fr)).cpu().numpy(), ref) < tol
    assert rel_l2(p.execute(torch.from_numpy(fr), real_out=True).cpu().numpy(), ref.real) < tol
    got = p.execute(torch.from_numpy(np.fft.ifftshift(fr)), real_out=True, fft_order=True).cpu().numpy()
    assert rel_l2(got, ref.real) < tol


def test_support_and_scale(nf):
    rng = np.random.default_rng(9)
    M, N = 13, 5000
    x, y, z = _pts(rng, N)
    sup = (rng.random((M,) * 3) > 0.4).astype(np.float32)
    c = rng.standard_normal(N).astype(np.float32)
    ref = on.type1(x, y, z, c, M, eps=1e-13) * sup / M ** 3
    p = nf.Plan(1, M).set_pts(torch.from_numpy(x), torch.from_numpy(y), torch.from_numpy(z))
    got = p.execute(torch.from_numpy(c), support=torch.from_numpy(sup), scale=1.0 / M ** 3, real_out=True)
    assert rel_l2(got.cpu().numpy(), ref.real) < TOL32


def test_reference_wrappers_fixture(nf, golden):
    g = golden("nufft_wrappers")
    ug = g["ugrid"].copy()
    fwd = nf.forward_gpu(ug, g["H"], g["K"], g["L"], g["support"], True)
    assert np.array_equal(ug, g["ugrid"] * g["support"])  # in-place support, forward.py:67-68
    assert fwd.dtype == np.complex64 and rel_l2(fwd, g["forward"]) < TOL32
    M = int(g["M"])
    adj = nf.adjoint_gpu(g["nuvect"], g["H"], g["K"], g["L"], M, True, g["support"])
    assert adj.shape == (M,) * 3 and rel_l2(adj, g["adjoint"]) < TOL32
    adjc = nf.adjoint_gpu(g["nuvect"], g["H"], g["K"], g["L"], M, False, None)
    assert np.iscomplexobj(adjc) and rel_l2(adjc, g["adjoint_complex"]) < TOL32


def test_range_assertion(nf):
    x = np.zeros(10, np.float32)
    x[3] = 3.0 * np.pi + 0.01
    with pytest.raises(AssertionError):
        nf.forward_gpu(np.ones((5, 5, 5), np.float32), x, x * 0, x * 0)


def test_quaternion_points_match_reference_chain(nf):
    from cmtip_gb300 import geometry
    rng = np.random.default_rng(5)
    ppr, rext = geometry.ewald_detector(16)
    rext = rext / 0.9
    quats = geometry.random_quaternions(7, rng).astype(np.float32)
    M = 21
    f = rng.standard_normal((M,) * 3)
    H, K, L = rp.gen_nonuniform_positions(quats, ppr)
    xs = [a.astype(np.float32).ravel() / rext * np.pi for a in (H, K, L)]
    ref = on.type2(*xs, f, eps=1e-13, isign=-1).real
    p = nf.Plan(2, M, isign=-1)
    p.set_pts_quat(nf.inverse_rotations(quats), torch.from_numpy(ppr.reshape(3, -1)), rext)
    got = p.execute(torch.from_numpy(f), real_out=True).cpu().numpy()
    assert rel_l2(got, ref) < TOL32
    inv = nf.inverse_rotations(quats).cpu().numpy()
    assert np.allclose(inv, np.linalg.inv(geometry.quaternion2rot3d(quats)), rtol=0, atol=1e-15)


def test_quaternion_coordinates_equal_float64_chain(nf):
    # An FP32 plan's quaternion points evaluate the float64 chain float32(inv(R) . p), then
    # / extent * pi, at FP32 throughput (a compensated dot product).  A type-2 output depends
    # only on its point's coordinates, so against the same plan fed the float64 chain's
    # float32 coordinates the outputs are bit-equal wherever the coordinates are; the two
    # may differ only for a value within ~2^-46 of a float32 rounding boundary (about one
    # coordinate in 10^7).
    from cmtip_gb300 import geometry
    rng = np.random.default_rng(8)
    ppr, rext = geometry.ewald_detector(64)
    rext = rext / 0.9
    quats = geometry.random_quaternions(64, rng).astype(np.float32)
    inv = nf.inverse_rotations(quats)
    R = inv.cpu().numpy().reshape(-1, 3, 3)
    pp = ppr.reshape(3, -1)
    xs = [np.ascontiguousarray(((R[:, r, 0, None] * pp[0] + R[:, r, 1, None] * pp[1]) + R[:, r, 2, None] * pp[2])
                               .astype(np.float32).astype(np.float64).ravel() / rext * np.pi).astype(np.float32)
          for r in range(3)]
    M = 41
    f = torch.from_numpy(rng.standard_normal((M,) * 3).astype(np.float32)).cuda()
    p = nf.Plan(2, M, isign=-1)
    p.set_pts(*(torch.from_numpy(a).cuda() for a in xs))
    ref = p.execute(f, real_out=True).cpu().numpy()
    p.set_pts_quat(inv, torch.from_numpy(pp).cuda(), rext)
    got = p.execute(f, real_out=True).cpu().numpy()
    p.close()
    assert got.size == 64 * pp.shape[1]
    assert np.count_nonzero(got != ref) <= 8
    assert rel_l2(got, ref) < 1e-6


@pytest.mark.parametrize("prec", [32, 64])
def test_derived_plan_on_twice_finer_grid(nf, prec):
    # the 2M-mode plan borrowing an M-mode plan's sorted points equals an independent plan
    rng = np.random.default_rng(21)
    M, N = 17, 20000
    x, y, z = _pts(rng, N)
    c = rng.standard_normal(N)
    eps, tol = (1e-6, TOL32) if prec == 32 else (1e-12, TOL64)
    src = nf.Plan(1, M, eps=eps, isign=1, prec=prec).set_pts(*(torch.from_numpy(a) for a in (x, y, z)))
    d = src.derive(1, 2 * M, isign=1)
    assert d.info()["n_fine"] == 2 * src.info()["n_fine"]
    ref = on.type1(x, y, z, c, 2 * M, eps=1e-13, isign=1)
    got = d.execute(torch.from_numpy(c), real_out=True, fft_order=True, scale=0.5)
    assert rel_l2(got.cpu().numpy(), 0.5 * np.fft.ifftshift(ref.real)) < tol
    assert rel_l2(d.execute(None, real_out=True).cpu().numpy(),
                  on.type1(x, y, z, np.ones(N), 2 * M, eps=1e-13).real) < tol
    # complex strengths through the extended window as well
    cc = c + 1j * rng.standard_normal(N)
    assert rel_l2(d.execute(torch.from_numpy(cc)).cpu().numpy(), on.type1(x, y, z, cc, 2 * M, eps=1e-13)) < tol
    # new points on the source are followed by the derived plan
    x2 = x[::-1].copy()
    src.set_pts(*(torch.from_numpy(a) for a in (x2, y, z)))
    assert rel_l2(d.execute(torch.from_numpy(c)).cpu().numpy(), on.type1(x2, y, z, c, 2 * M, eps=1e-13)) < tol


@pytest.mark.parametrize("prec,eps", [(32, 1e-3), (32, 1e-4), (32, 1e-5), (32, 1e-6), (64, 1e-6), (64, 1e-5)])
def test_derived_extended_window_matches_plain(nf, prec, eps, monkeypatch):
    # widths 4..7: real spreading on the derived grid through the (w+1)^3 register window
    # equals the per-origin kernel and the oracle
    rng = np.random.default_rng(22)
    M, N = 19, 30000
    x, y, z = _pts(rng, N)
    c = rng.standard_normal(N)
    src = nf.Plan(1, M, eps=eps, isign=1, prec=prec).set_pts(*(torch.from_numpy(a) for a in (x, y, z)))
    ext = src.derive(1, 2 * M, isign=1)
    monkeypatch.setenv("CMT_SPREAD_EXT", "0")
    plain = src.derive(1, 2 * M, isign=1)
    a = ext.execute(torch.from_numpy(c), real_out=True).cpu().numpy()
    b = plain.execute(torch.from_numpy(c), real_out=True).cpu().numpy()
    assert rel_l2(a, b) < (1e-6 if prec == 32 else 1e-13)
    ref = on.type1(x, y, z, c, 2 * M, eps=1e-13, isign=1).real
    assert rel_l2(a, ref) < 20 * eps


@pytest.mark.parametrize("prec,eps", [(32, 1e-2), (32, 1e-4), (32, 1e-6), (64, 1e-7), (64, 1e-5)])
@pytest.mark.parametrize("cplx", [False, True])
def test_table_spread_matches_per_point_kernel(nf, prec, eps, cplx, monkeypatch):
    # widths 3..8: the table-driven spreading kernel equals the per-point kernel and the oracle
    rng = np.random.default_rng(23)
    M, N = 24, 40000
    x, y, z = _pts(rng, N)
    c = rng.standard_normal(N) + (1j * rng.standard_normal(N) if cplx else 0)
    pts = [torch.from_numpy(a) for a in (x, y, z)]
    tab = nf.Plan(1, M, eps=eps, isign=1, prec=prec).set_pts(*pts)
    monkeypatch.setenv("CMT_SPREAD_TAB", "0")
    ref_plan = nf.Plan(1, M, eps=eps, isign=1, prec=prec).set_pts(*pts)
    a = tab.execute(torch.from_numpy(c)).cpu().numpy()
    b = ref_plan.execute(torch.from_numpy(c)).cpu().numpy()
    assert rel_l2(a, b) < (1e-6 if prec == 32 else 1e-13)
    assert rel_l2(a, on.type1(x, y, z, c, M, eps=1e-13, isign=1)) < max(20 * eps, 1e-5)


@pytest.mark.parametrize("prec,eps", [(32, 1e-2), (32, 1e-4), (32, 1e-6), (64, 1e-7), (64, 1e-5)])
@pytest.mark.parametrize("real_out", [False, True])
def test_table_interp_matches_per_point_kernel(nf, prec, eps, real_out, monkeypatch):
    # widths 3..8: the table-driven interpolation kernel equals the per-point kernel and the
    # oracle, complex output from the complex grid and real output from the real grid
    rng = np.random.default_rng(24)
    M, N = 24, 40000
    x, y, z = _pts(rng, N)
    f = rng.standard_normal((M,) * 3) + 1j * rng.standard_normal((M,) * 3)
    pts = [torch.from_numpy(a) for a in (x, y, z)]
    tab = nf.Plan(2, M, eps=eps, isign=-1, prec=prec).set_pts(*pts)
    monkeypatch.setenv("CMT_INTERP_TAB", "0")
    ref_plan = nf.Plan(2, M, eps=eps, isign=-1, prec=prec).set_pts(*pts)
    a = tab.execute(torch.from_numpy(f), real_out=real_out).cpu().numpy()
    b = ref_plan.execute(torch.from_numpy(f), real_out=real_out).cpu().numpy()
    assert rel_l2(a, b) < (1e-6 if prec == 32 else 1e-13)
    ref = on.type2(x, y, z, f, eps=1e-13, isign=-1)
    assert rel_l2(a, ref.real if real_out else ref) < max(20 * eps, 1e-5)


@pytest.mark.parametrize("prec", [32, 64])
def test_plan_repointed_with_growing_and_shrinking_point_sets(nf, prec):
    # one plan (and a derived plan on its points) set to 20k, 90k, then 5k points: the sort's
    # buffers grow from the stream-ordered pool and are reused; every execute matches the
    # oracle for the points it was given last
    rng = np.random.default_rng(31)
    M = 17
    eps, tol = (1e-6, TOL32) if prec == 32 else (1e-12, TOL64)
    p = nf.Plan(1, M, eps=eps, isign=1, prec=prec)
    d = p.derive(1, 2 * M, isign=1)
    q = nf.Plan(2, M, eps=eps, isign=-1, prec=prec)
    f = rng.standard_normal((M,) * 3)
    for N in (20000, 90000, 5000):
        x, y, z = _pts(rng, N)
        c = rng.standard_normal(N)
        pts = [torch.from_numpy(a) for a in (x, y, z)]
        p.set_pts(*pts)
        q.set_pts(*pts)
        assert rel_l2(p.execute(torch.from_numpy(c)).cpu().numpy(), on.type1(x, y, z, c, M, eps=1e-13)) < tol
        assert rel_l2(d.execute(None, real_out=True).cpu().numpy(),
                      on.type1(x, y, z, np.ones(N), 2 * M, eps=1e-13).real) < tol
        assert rel_l2(q.execute(torch.from_numpy(f)).cpu().numpy(), on.type2(x, y, z, f, eps=1e-13, isign=-1)) < tol
    d.close()
    p.close()
    q.close()


@pytest.mark.parametrize("prec", [32, 64])
def test_pair_is_normal_operator(nf, prec):
    rng = np.random.default_rng(11)
    M, N = 15, 30000
    x, y, z = _pts(rng, N)
    f = rng.standard_normal((M,) * 3)
    sup = (rng.random((M,) * 3) > 0.2).astype(np.float32)
    c = on.type2(x, y, z, f * sup, eps=1e-13, isign=-1)
    ref = (on.type1(x, y, z, c, M, eps=1e-13, isign=1).real * sup) / (2 * M) ** 3
    p = nf.Plan(1, M, isign=1, prec=prec, eps=1e-6 if prec == 32 else 1e-12)
    p.set_pts(torch.from_numpy(x), torch.from_numpy(y), torch.from_numpy(z))
    got = p.execute_pair(torch.from_numpy(f), support=torch.from_numpy(sup), scale=1.0 / (2 * M) ** 3)
    assert rel_l2(got.cpu().numpy(), ref) < (TOL32 if prec == 32 else TOL64)


@pytest.mark.parametrize("prec,eps", [(32, 1e-2), (32, 1e-4), (32, 1e-6), (64, 1e-7), (64, 1e-5)])
@pytest.mark.parametrize("tuning", [None, (5, 2048)])
def test_table_pair_matches_per_point_pair(nf, prec, eps, tuning, monkeypatch):
    # widths 3..8: the table-driven fused pair (kernel values once per point for both
    # directions) equals the per-point pair and the exact normal operator
    rng = np.random.default_rng(25)
    M, N = 21, 40000
    x, y, z = _pts(rng, N)
    f = rng.standard_normal((M,) * 3)
    sup = (rng.random((M,) * 3) > 0.2).astype(np.float32)
    pts = [torch.from_numpy(a) for a in (x, y, z)]

    def plan():
        p = nf.Plan(1, M, eps=eps, isign=1, prec=prec)
        if tuning:
            p.set_tuning(*tuning)
        return p.set_pts(*pts)
    tab = plan()
    monkeypatch.setenv("CMT_INTERP_TAB", "0")
    ref_plan = plan()
    a = tab.execute_pair(torch.from_numpy(f), support=torch.from_numpy(sup)).cpu().numpy()
    b = ref_plan.execute_pair(torch.from_numpy(f), support=torch.from_numpy(sup)).cpu().numpy()
    assert rel_l2(a, b) < (1e-6 if prec == 32 else 1e-13)
    c = on.type2(x, y, z, f * sup, eps=1e-13, isign=-1)
    ref = on.type1(x, y, z, c, M, eps=1e-13, isign=1).real * sup
    assert rel_l2(a, ref) < max(40 * eps, 1e-5)


def test_adjointness_large(nf):
    # <A f, c> == <f, A^H c> at 4M points with FP32 kernels, FP64 inner products
    rng = np.random.default_rng(12)
    M, N = 41, 4_000_000
    g = torch.Generator(device="cuda").manual_seed(1)
    x, y, z = [(torch.rand(N, device="cuda", generator=g) * 2 - 1) * np.pi for _ in range(3)]
    f = torch.randn((M,) * 3, device="cuda", dtype=torch.complex64, generator=g)
    c = torch.randn(N, device="cuda", dtype=torch.complex64, generator=g)
    A = nf.Plan(2, M, isign=-1).set_pts(x, y, z)
    AH = nf.Plan(1, M, isign=1).set_pts(x, y, z)
    lhs = torch.vdot(c.to(torch.complex128), A.execute(f).to(torch.complex128))
    rhs = torch.vdot(AH.execute(c).to(torch.complex128).reshape(-1), f.to(torch.complex128).reshape(-1))
    assert abs(complex(lhs) - complex(rhs)) / abs(complex(lhs)) < 1e-5
