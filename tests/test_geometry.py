"""Host geometry on CPU: rotation matrices, quaternion samplers, the Ewald-sphere detector
and the synthetic particle's autocorrelation (the bit-exact match of the reference's
position chain is in test_oracle.py)."""
import numpy as np

from cmtip_gb300 import geometry


def test_rotations_are_proper_and_follow_the_w_x_y_z_convention():
    rng = np.random.default_rng(1)
    q = geometry.random_quaternions(500, rng)
    R = geometry.quaternion2rot3d(q)
    assert R.shape == (500, 3, 3) and R.dtype == np.float64
    assert np.allclose(R @ R.transpose(0, 2, 1), np.eye(3), atol=1e-12)
    assert np.allclose(np.linalg.det(R), 1.0, atol=1e-12)
    assert np.array_equal(geometry.quaternion2rot3d(np.array([1.0, 0, 0, 0])), np.eye(3))
    t = 0.7  # (cos t/2, 0, 0, sin t/2): rotation by t about z
    Rz = geometry.quaternion2rot3d(np.array([np.cos(t / 2), 0, 0, np.sin(t / 2)]))
    assert np.allclose(Rz, [[np.cos(t), -np.sin(t), 0], [np.sin(t), np.cos(t), 0], [0, 0, 1]], atol=1e-15)
    assert np.allclose(geometry.quaternion2rot3d(-q), R)  # q and -q: one rotation
    assert np.allclose(geometry.inverse_rotations(q), R.transpose(0, 2, 1), atol=1e-12)


def test_quaternion_samplers():
    for q in (geometry.uniform_quaternions(2000), geometry.random_quaternions(2000, np.random.default_rng(3))):
        assert q.shape == (2000, 4)
        assert np.allclose(np.linalg.norm(q, axis=1), 1.0, atol=1e-12)
        assert (q[:, 0] >= 0).all()
    a = geometry.random_quaternions(10, np.random.default_rng(5))
    assert np.array_equal(a, geometry.random_quaternions(10, np.random.default_rng(5)))
    # uniform on SO(3): the rotation angle 2 acos(w) has density (1 - cos a) / pi on [0, pi],
    # so its mean is pi/2 + 2/pi
    for q in (geometry.uniform_quaternions(20000), geometry.random_quaternions(20000, np.random.default_rng(7))):
        ang = 2 * np.arccos(np.clip(q[:, 0], -1, 1))
        assert abs(ang.mean() - (np.pi / 2 + 2 / np.pi)) < 0.02


def test_ewald_detector_lies_on_the_sphere():
    lam = 2.5e-10
    ppr, rext = geometry.ewald_detector(16, wavelength=lam)
    assert ppr.shape == (3, 1, 4 * 16 * 16)
    q = ppr.reshape(3, -1)
    # q = (n - z) / lambda with |n| = 1: |lambda q + z| = 1
    assert np.allclose(np.linalg.norm(lam * q + np.array([[0], [0], [1.0]]), axis=0), 1.0, atol=1e-12)
    assert rext == np.linalg.norm(q, axis=0).max()
    assert (q[2] < 0).all()  # q_z = (n_z - 1) / lambda < 0 off the beam axis
    # four panels, one per quadrant of the detector plane
    assert sorted(set(zip(np.sign(q[0]), np.sign(q[1])))) == [(-1, -1), (-1, 1), (1, -1), (1, 1)]


def test_particle_autocorrelation_is_centrosymmetric_and_sums_to_mass_squared():
    rng = np.random.default_rng(2)
    M = 21
    rho = geometry.gaussian_particle(M, 12, 4.0, rng)
    assert rho.shape == (M,) * 3 and (rho >= 0).all()
    ac = geometry.autocorrelation_of(rho)
    assert np.allclose(ac, ac[::-1, ::-1, ::-1], atol=1e-12 * ac.max())
    assert np.isclose(ac.sum(), rho.sum() ** 2, rtol=1e-12)
    assert np.unravel_index(ac.argmax(), ac.shape) == (M // 2,) * 3
