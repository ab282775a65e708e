"""ORACLE (test infrastructure only): numpy restatement of cmtip's hot path.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline /
reference legs may import this module; the product never does.

Each function restates one reference function (file:line in the cmtip project) with
the same arithmetic and dtype behaviour; the finufft calls are served by the FP64
oracle NUFFT in ``oracle/nufft.py`` and skopi's quaternion helpers by
``cmtip_gb300.geometry`` (skopi is not available).  The restatement is pinned against
golden fixtures produced by importing the unmodified reference
(``tests/golden/make_golden.py``).
"""
from __future__ import annotations

import numpy as np
from scipy.ndimage import gaussian_filter
from scipy.sparse.linalg import LinearOperator, cg

from cmtip_gb300.geometry import quaternion2rot3d, uniform_quaternions
from oracle import nufft as onufft

NUFFT_EPS = 1e-12


# ---------------------------------------------------------------- cmtip/nufft

def forward_cpu(ugrid, H_, K_, L_, support=None, use_recip_sym=True, eps=NUFFT_EPS, out_dtype=np.complex64):
    """cmtip/nufft/forward.py:13-42: type 2, isign=-1, optional support (in place), complex64 out."""
    H_, K_, L_ = (np.asarray(a) for a in (H_, K_, L_))
    assert np.max(np.abs(np.array([H_, K_, L_]))) < 3 * np.pi
    if use_recip_sym:
        assert np.all(np.isreal(ugrid))
    if support is not None:
        ugrid *= support
    c = onufft.type2(H_, K_, L_, np.asarray(ugrid, dtype=np.complex128), eps=eps, isign=-1)
    return c.reshape(H_.shape).astype(out_dtype)


def adjoint_cpu(nuvect, H_, K_, L_, M, use_recip_sym=True, support=None, eps=NUFFT_EPS,
                grid_dtype=np.complex64):
    """cmtip/nufft/adjoint.py:13-43: type 1, isign=+1, complex64 grid, *support, .real, / M^3."""
    H_, K_, L_ = (np.asarray(a) for a in (H_, K_, L_))
    assert np.max(np.abs(np.array([H_, K_, L_]))) < 3 * np.pi
    ugrid = onufft.type1(H_, K_, L_, np.asarray(nuvect), M, eps=eps, isign=1).astype(grid_dtype)
    if support is not None:
        ugrid = ugrid * support
    if use_recip_sym:
        ugrid = ugrid.real
    return ugrid / (M ** 3)


# ------------------------------------------------------ cmtip/autocorrelation

def gen_nonuniform_positions(orientations, pixel_position_reciprocal):
    """autocorrelation.py:12-29: H,K,L = inv(R(q)) . ppr, float64 (n_img, n_panels, n_pix)."""
    if orientations.shape[0] > 0:
        rotmat = np.array([np.linalg.inv(quaternion2rot3d(q)) for q in orientations])
    else:
        rotmat = np.eye(3)[None]
    HKL = np.einsum("ijk,klm->jilm", rotmat, pixel_position_reciprocal)
    return HKL[0], HKL[1], HKL[2]


def core_problem_convolution(uvect, M, F_ugrid_conv_, M_ups, ac_support, use_recip_sym=True):
    """autocorrelation.py:32-63: support, zero-pad to M_ups^3 corner, FFT-multiply, crop."""
    if use_recip_sym:
        assert np.all(np.isreal(uvect))
    padded = np.zeros((M_ups,) * 3, dtype=uvect.dtype)
    padded[:M, :M, :M] = uvect.reshape((M,) * 3) * ac_support
    spec = np.fft.fftn(np.fft.ifftshift(padded)) * F_ugrid_conv_
    conv = np.fft.fftshift(np.fft.ifftn(spec))[:M, :M, :M] * ac_support
    if use_recip_sym:
        conv = conv.real
    return conv.flatten()


def gen_F_antisupport(M):
    """autocorrelation.py:66-85: |q| > pi on linspace(-pi, pi, M)^3, |q| rounded to 4 dp."""
    lu = np.linspace(-np.pi, np.pi, M)
    q2 = lu[:, None, None] ** 2 + lu[None, :, None] ** 2 + lu[None, None, :] ** 2
    return np.around(np.sqrt(q2), 4) > np.pi


def fourier_reg(uvect, support, F_antisupport, M, use_recip_sym):
    """autocorrelation.py:88-110: support, FFT, zero the central sphere, IFFT, support."""
    grid = uvect.reshape((M,) * 3) * support
    if use_recip_sym:
        assert np.all(np.isreal(grid))
    spec = np.fft.fftn(np.fft.ifftshift(grid)) * np.fft.ifftshift(F_antisupport)
    out = (np.fft.fftshift(np.fft.ifftn(spec)) * support).flatten()
    return out.real if use_recip_sym else out


def setup_linops(H, K, L, data, ac_support, weights, x0, M, Mtot, N, reciprocal_extent,
                 alambda, rlambda, flambda, use_recip_sym=True, eps=NUFFT_EPS):
    """autocorrelation.py:113-173: W = a*ADA(Toeplitz, 2M grid) + r*I + f*FDF; d = a*A^H(Db) + r*x0."""
    H_ = H.flatten() / reciprocal_extent * np.pi
    K_ = K.flatten() / reciprocal_extent * np.pi
    L_ = L.flatten() / reciprocal_extent * np.pi
    F_antisupport = gen_F_antisupport(M)
    M_ups = 2 * M
    kern = adjoint_cpu(np.ones_like(data, dtype=np.complex64), H_, K_, L_, M_ups,
                       use_recip_sym=use_recip_sym, support=None, eps=eps)
    F_ugrid_conv_ = np.fft.fftn(np.fft.ifftshift(kern))

    def matvec(u):
        ada = core_problem_convolution(u, M, F_ugrid_conv_, M_ups, ac_support)
        fdf = fourier_reg(u, ac_support, F_antisupport, M, use_recip_sym=use_recip_sym)
        return alambda * ada + rlambda * u + flambda * fdf

    W = LinearOperator(dtype=np.complex64, shape=(Mtot, Mtot), matvec=matvec)
    nuvect_Db = (data * weights).astype(np.complex64)
    ADb = adjoint_cpu(nuvect_Db, H_, K_, L_, M, support=ac_support,
                      use_recip_sym=use_recip_sym, eps=eps).flatten()
    d = alambda * ADb + rlambda * x0
    return W, d, F_ugrid_conv_


def solve_ac_inputs(pixel_position_reciprocal, slices_, M, orientations, ac_estimate):
    """autocorrelation.py:199-226: positions, support, lambdas (shared by solve_ac and tests)."""
    Mtot = M ** 3
    N = np.prod(slices_.shape)  # numpy int64 (autocorrelation.py:201): rlambda and d become float64
    H, K, L = gen_nonuniform_positions(orientations, pixel_position_reciprocal)
    H, K, L = H.astype(np.float32), K.astype(np.float32), L.astype(np.float32)
    data = slices_.flatten().astype(np.float32)
    if ac_estimate is None:
        ac_support = np.ones((M,) * 3)
        ac_estimate = np.zeros((M,) * 3)
    else:
        ac_support = (gaussian_filter(ac_estimate, 0.5) > 1e-12).astype(np.float32)
        ac_estimate = ac_estimate * ac_support
    weights = np.ones(N).astype(np.float32)
    return dict(H=H, K=K, L=L, data=data, ac_support=ac_support, x0=ac_estimate.flatten(),
                weights=weights, alambda=1, rlambda=Mtot / N / 1000, flambda=1e3, Mtot=Mtot, N=N)


def solve_ac(pixel_position_reciprocal, reciprocal_extent, slices_, M, orientations,
             ac_estimate=None, maxiter=100, rtol=1e-5, use_recip_sym=True, eps=NUFFT_EPS):
    """autocorrelation.py:176-248 with explicit maxiter/rtol (the reference hard-codes 100 / 1e-5).

    Returns (ac float64 (M,M,M), iterations)."""
    s = solve_ac_inputs(pixel_position_reciprocal, slices_, M, orientations, ac_estimate)
    W, d, _ = setup_linops(s["H"], s["K"], s["L"], s["data"], s["ac_support"], s["weights"], s["x0"],
                           M, s["Mtot"], s["N"], reciprocal_extent, s["alambda"], s["rlambda"],
                           s["flambda"], use_recip_sym=use_recip_sym, eps=eps)
    count = [0]
    ret, info = cg(W, d, x0=s["x0"], maxiter=maxiter, rtol=rtol, callback=lambda xk: count.__setitem__(0, count[0] + 1))
    return ret.reshape((M,) * 3).real, count[0]


# ------------------------------------------------------------ cmtip/alignment

def generate_weights(pixel_position_reciprocal, order=0):
    """align.py:11-24: 1/|s|^order (s in 1/Angstrom) normalised to sum 1."""
    s = np.linalg.norm(pixel_position_reciprocal, axis=0) * 1e-10
    w = 1.0 / (s ** order)
    return w / np.sum(w)


def calc_eudist(model_slices, slices):
    """align.py:27-36 (sklearn euclidean_distances): sqrt(max(|a|^2 + |b|^2 - 2 a.b, 0)) in float64."""
    a = np.asarray(model_slices, dtype=np.float64)
    b = np.asarray(slices, dtype=np.float64)
    d2 = (a * a).sum(1)[:, None] - 2.0 * a @ b.T + (b * b).sum(1)[None, :]
    return np.sqrt(np.maximum(d2, 0.0))


def compute_slices(orientations, pixel_position_reciprocal, reciprocal_extent, ac, eps=NUFFT_EPS):
    """align.py:39-65: rotate, float32 cast, scale by pi/reciprocal_extent, type 2, real part."""
    rotmat = np.array([np.linalg.inv(quaternion2rot3d(q)) for q in orientations])
    H, K, L = np.einsum("ijk,klm->jilm", rotmat, pixel_position_reciprocal)
    H_ = H.astype(np.float32).flatten() / reciprocal_extent * np.pi
    K_ = K.astype(np.float32).flatten() / reciprocal_extent * np.pi
    L_ = L.astype(np.float32).flatten() / reciprocal_extent * np.pi
    return forward_cpu(ac, H_, K_, L_, support=None, use_recip_sym=True, eps=eps).real


def reference_orientations(n_ref_orientations, nbatches=1, true_orientations=None, ref_orientations=None,
                           shuffle_rng=None):
    """align.py:96-111: pad n_ref to a multiple of nbatches, uniform quaternions (float32),
    optionally splice in true orientations and shuffle."""
    quot, rem = divmod(n_ref_orientations, nbatches)
    if rem != 0:
        n_ref_orientations = (quot + 1) * nbatches
    if ref_orientations is None:
        ref_orientations = uniform_quaternions(n_ref_orientations)
    ref = np.asarray(ref_orientations).astype(np.float32)
    if true_orientations is not None:
        ref = np.vstack((ref[:-len(true_orientations)], true_orientations))
        (shuffle_rng or np.random).shuffle(ref)
    return ref


def match_orientations(pixel_position_reciprocal, reciprocal_extent, slices_, ac, ref_orientations,
                       nbatches=1, order=0, eps=NUFFT_EPS, return_distances=False):
    """align.py:68-132 on given reference orientations: per-batch std scaling, weighted
    euclidean distances, argmin over references.  Returns (matched quats, index[, distances])."""
    n_ref = ref_orientations.shape[0]
    quot = n_ref // nbatches
    n_pix = pixel_position_reciprocal.shape[-1]
    slices_ = slices_.reshape((slices_.shape[0], n_pix))
    distances = np.zeros((n_ref, slices_.shape[0]))
    weights = generate_weights(pixel_position_reciprocal, order=order)
    for nb in range(nbatches):
        start, end = nb * quot, (nb + 1) * quot
        model = compute_slices(ref_orientations[start:end], pixel_position_reciprocal, reciprocal_extent,
                               ac, eps=eps).reshape((end - start, n_pix))
        model *= slices_.std() / model.std()
        distances[start:end, :] = calc_eudist(model * weights, slices_ * weights)
    index = np.argmin(distances, axis=0)
    if return_distances:
        return ref_orientations[index], index, distances
    return ref_orientations[index], index


def match_orientations_mult(pixel_position_reciprocal, reciprocal_extent, slices_, ac_mult, ref_orientations,
                            nbatches=1, order=0, eps=NUFFT_EPS):
    """align.py:135-213 on given reference orientations: every image matched against each
    volume (match_orientations per volume), then the volume with the smallest best distance
    (first index on ties) and that volume's best reference.  Returns (quats, conformations)."""
    n_img = slices_.shape[0]
    indices = np.zeros((len(ac_mult), n_img), dtype=np.int64)
    min_dists = np.zeros((len(ac_mult), n_img))
    for k, ac in enumerate(ac_mult):
        _, idx, dist = match_orientations(pixel_position_reciprocal, reciprocal_extent, slices_, ac,
                                          ref_orientations, nbatches=nbatches, order=order, eps=eps,
                                          return_distances=True)
        indices[k], min_dists[k] = idx, dist.min(axis=0)
    conformations = np.argmin(min_dists, axis=0)
    index = indices[conformations, np.arange(n_img)]
    return ref_orientations[index], conformations


# ------------------------------------------------------------ cmtip/phasing

def phase_recenter_grid(M):
    """phase.py:34-38: per-axis midpoints of linspace(-1, 1, M + 1) on an ij mesh, each
    coordinate ifftshifted; shape (3, M, M, M)."""
    edges = np.linspace(-1, 1, M + 1)
    mids = (edges[:-1] + edges[1:]) / 2
    return np.stack([np.fft.ifftshift(c) for c in np.meshgrid(mids, mids, mids, indexing="ij")])


def phase_center_of_mass(rho_, hkl_, M):
    """phase.py:11-23: rounded |rho_|-weighted mean of hkl_, in voxels (M / 2 per unit)."""
    w = np.abs(rho_)
    return np.round((w * hkl_).sum(axis=(1, 2, 3)) / w.sum() * M / 2)


def phase_recenter(rho_, support_, M):
    """phase.py:26-44: roll both arrays (in place) by minus the centre of mass, axis by axis."""
    shifts = phase_center_of_mass(rho_, phase_recenter_grid(M), M)
    for axis in range(3):
        s = int(shifts[axis])
        rho_[:] = np.roll(rho_, -s, axis)
        support_[:] = np.roll(support_, -s, axis)


def phase_create_support(ac_, M, Mquat):
    """phase.py:47-64: centred cube [Mquat, M - Mquat)^3 (ifftshifted) and ac_ above 1% of its max."""
    cube = np.zeros((M, M, M), dtype=np.bool_)
    cube[Mquat:M - Mquat, Mquat:M - Mquat, Mquat:M - Mquat] = Mquat > 0
    return np.fft.ifftshift(cube) & (ac_ > 1e-2 * ac_.max())


def phase_amplitudes(ac):
    """phase.py:186-192: ac_filt_ (ifftshifted Gaussian-filtered positive part) and
    amplitudes_ = sqrt(|fftn(ac_filt_)|)."""
    filt = gaussian_filter(np.maximum(ac.real, 0), mode="constant", sigma=1, truncate=2)
    ac_filt_ = np.fft.ifftshift(filt)
    return ac_filt_, np.sqrt(np.abs(np.fft.fftn(ac_filt_)))


def phase_step(rho_, amplitudes_, amp_mask_, support_):
    """phase.py:122-144: replace the masked Fourier moduli by amplitudes_, keep the phases,
    back-transform (real part) and intersect the support with positivity."""
    spec = np.fft.fftn(rho_)
    spec = np.where(amp_mask_, amplitudes_ * np.exp(1j * np.angle(spec)), spec)
    rho_mod_ = np.fft.ifftn(spec).real
    return rho_mod_, np.logical_and(support_, rho_mod_ > 0)


def phase_er(rho_, amplitudes_, amp_mask_, support_, rho_max, n_loops=1):
    """phase.py:67-72, 83-99: Error Reduction, rho_ in place."""
    for _ in range(n_loops):
        rho_mod_, star = phase_step(rho_, amplitudes_, amp_mask_, support_)
        rho_[:] = np.where(star, rho_mod_, 0)
        rho_[rho_mod_ > rho_max] = rho_max


def phase_hio(beta, rho_, amplitudes_, amp_mask_, support_, rho_max, n_loops=1):
    """phase.py:75-80, 102-119: Hybrid Input-Output, rho_ in place."""
    for _ in range(n_loops):
        rho_mod_, star = phase_step(rho_, amplitudes_, amp_mask_, support_)
        rho_[:] = np.where(star, rho_mod_, rho_ - beta * rho_mod_)
        over = rho_mod_ > rho_max
        rho_[over] += 2 * beta * rho_mod_[over] - rho_max


def phase_shrink_wrap(cutoff, sigma, rho_, support_):
    """phase.py:147-162: support_ (in place) where the periodic Gaussian-smoothed |rho_|
    exceeds cutoff * max|rho_|."""
    a = np.absolute(rho_)
    support_[:] = gaussian_filter(a, mode="wrap", sigma=sigma, truncate=2) > a.max() * cutoff


def phase(generation, ac, support_=None, rho_=None, n_iterations=10, nER=50, nHIO=25):
    """phase.py:165-219: ER / HIO(0.3) / ER / shrink-wrap(5e-2, 1) cycles, a final ER loop,
    recentring, and fftshift(|ifftn(|fftn(rho_)|^2)|).  The random start uses numpy's
    global generator, as the reference's."""
    M = ac.shape[0]
    Mquat = int((M - 1) / 4)
    ac_filt_, amplitudes_ = phase_amplitudes(ac)
    amp_mask_ = np.ones((M, M, M), dtype=np.bool_)
    amp_mask_[0, 0, 0] = False
    if support_ is None:
        support_ = phase_create_support(ac_filt_, M, Mquat)
    if rho_ is None:
        rho_ = support_ * np.random.rand(*support_.shape)
    for _ in range(n_iterations):
        phase_er(rho_, amplitudes_, amp_mask_, support_, np.inf, nER)
        phase_hio(0.3, rho_, amplitudes_, amp_mask_, support_, np.inf, nHIO)
        phase_er(rho_, amplitudes_, amp_mask_, support_, np.inf, nER)
        phase_shrink_wrap(5e-2, 1, rho_, support_)
    phase_er(rho_, amplitudes_, amp_mask_, support_, np.inf, nER)
    phase_recenter(rho_, support_, M)
    ac_phased_ = np.abs(np.fft.ifftn(np.abs(np.fft.fftn(rho_)) ** 2))
    return np.fft.fftshift(ac_phased_), support_, rho_
