"""Host-side geometry for single-particle imaging: quaternions, detector q-vectors,
seeded synthetic particles.

* ``quaternion2rot3d`` follows the batched restatement in the reference
  (``cmtip/eval/geom.py:25-46``, itself the skopi convention ``q = (w, x, y, z)``);
  element formulas are evaluated in the quaternion's own dtype (float32 quaternions
  give float32-rounded matrix entries, as skopi does), then stored as float64.
* ``uniform_quaternions`` replaces ``skopi.get_uniform_quat`` (called at
  ``cmtip/alignment/align.py:108``; skopi is not available here).  It is the
  super-Fibonacci spiral of Alexa (CVPR 2022), mapped to the ``w >= 0`` hemisphere
  because ``q`` and ``-q`` are the same rotation.
* ``random_quaternions`` replaces ``skopi.get_random_quat`` (``autocorrelation.py:207``):
  Shoemake's uniform sampling of unit quaternions from a seeded generator.
* ``ewald_detector`` builds a 4-panel flat detector and its reciprocal-space pixel
  positions on the Ewald sphere, shape ``(3, 1, n_pix)`` like the reference's
  ``pixel_position_reciprocal`` after reshaping to a monolithic detector.
* ``gaussian_particle`` / ``autocorrelation_of`` produce the seeded synthetic density
  (unit-weight isotropic Gaussians, sigma = 1 voxel, inside a sphere) and its
  autocorrelation on an ``M^3`` grid.
"""
from __future__ import annotations

import numpy as np


def quaternion2rot3d(quat):
    """Rotation matrices for quaternions ``(w, x, y, z)``; ``quat`` is (4,) or (n, 4)."""
    q = np.asarray(quat)
    single = q.ndim == 1
    if single:
        q = q[None, :]
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    rot = np.zeros((q.shape[0], 3, 3))
    rot[:, 0, 0] = 1.0 - 2.0 * (y * y + z * z)
    rot[:, 0, 1] = 2.0 * (x * y - w * z)
    rot[:, 0, 2] = 2.0 * (x * z + w * y)
    rot[:, 1, 0] = 2.0 * (x * y + w * z)
    rot[:, 1, 1] = 1.0 - 2.0 * (x * x + z * z)
    rot[:, 1, 2] = 2.0 * (y * z - w * x)
    rot[:, 2, 0] = 2.0 * (x * z - w * y)
    rot[:, 2, 1] = 2.0 * (y * z + w * x)
    rot[:, 2, 2] = 1.0 - 2.0 * (x * x + y * y)
    return rot[0] if single else rot


def inverse_rotations(quats):
    """``inv(quaternion2rot3d(q))`` per quaternion, float64 (n, 3, 3)."""
    return np.linalg.inv(quaternion2rot3d(np.asarray(quats)))


def uniform_quaternions(n: int) -> np.ndarray:
    """Deterministic, near-uniform quaternions on SO(3) (super-Fibonacci spiral), float64."""
    phi = np.sqrt(2.0)
    psi = 1.533751168755204288118041
    s = np.arange(n, dtype=np.float64) + 0.5
    t = s / n
    r = np.sqrt(t)
    R = np.sqrt(1.0 - t)
    alpha = 2.0 * np.pi * s / phi
    beta = 2.0 * np.pi * s / psi
    q = np.stack([r * np.sin(alpha), r * np.cos(alpha), R * np.sin(beta), R * np.cos(beta)], axis=1)
    q[q[:, 0] < 0] *= -1.0
    return q


def random_quaternions(n: int, rng) -> np.ndarray:
    """Uniform random unit quaternions (Shoemake 1992) from a numpy Generator."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    a, b = np.sqrt(1.0 - u1), np.sqrt(u1)
    q = np.stack([a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2),
                  b * np.sin(2 * np.pi * u3), b * np.cos(2 * np.pi * u3)], axis=1)
    q[q[:, 0] < 0] *= -1.0
    return q


def ewald_detector(P: int, wavelength: float = 2.5e-10, distance: float = 0.2,
                   half_width: float = 0.1, gap_pixels: float = 1.0):
    """Four P x P flat panels around the beam, pixel q-vectors on the Ewald sphere.

    Returns ``(ppr, reciprocal_extent)`` with ``ppr`` float64 of shape (3, 1, 4*P*P)
    in inverse metres and ``reciprocal_extent = max|q|`` (the reference's convention,
    ``cmtip/alignment/align.py:55-57``: coordinates are scaled by pi/reciprocal_extent).
    """
    pix = half_width / P
    c = (np.arange(P) + 0.5 + 0.5 * gap_pixels) * pix
    panels = []
    for sx in (-1.0, 1.0):
        for sy in (-1.0, 1.0):
            X, Y = np.meshgrid(sx * c, sy * c, indexing="ij")
            panels.append(np.stack([X.ravel(), Y.ravel()], 0))
    xy = np.concatenate(panels, axis=1)
    r = np.concatenate([xy, np.full((1, xy.shape[1]), distance)], axis=0)
    n = r / np.linalg.norm(r, axis=0, keepdims=True)
    q = (n - np.array([[0.0], [0.0], [1.0]])) / wavelength
    ppr = q.reshape(3, 1, -1)
    return ppr, float(np.linalg.norm(ppr, axis=0).max())


def gaussian_particle(M: int, n_atoms: int, radius: float, rng, sigma: float = 1.0):
    """Density on an M^3 grid: n_atoms unit-weight Gaussians uniform inside a sphere."""
    d = rng.standard_normal((n_atoms, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    pos = d * radius * rng.random(n_atoms)[:, None] ** (1.0 / 3.0)
    ax = np.arange(M) - M // 2
    rho = np.zeros((M, M, M))
    norm = (2 * np.pi * sigma ** 2) ** -1.5
    for p in pos:
        gx = np.exp(-0.5 * ((ax - p[0]) / sigma) ** 2)
        gy = np.exp(-0.5 * ((ax - p[1]) / sigma) ** 2)
        gz = np.exp(-0.5 * ((ax - p[2]) / sigma) ** 2)
        rho += norm * gx[:, None, None] * gy[None, :, None] * gz[None, None, :]
    return rho


def autocorrelation_of(rho):
    """Centred circular autocorrelation of a centred density (float64)."""
    F = np.fft.fftn(np.fft.ifftshift(rho))
    return np.fft.fftshift(np.fft.ifftn(np.abs(F) ** 2).real)
