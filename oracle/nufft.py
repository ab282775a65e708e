"""ORACLE (test infrastructure only): FP64 CPU 3D NUFFT and direct NUDFT.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may
import this module.  It checks results and is never on the product path.

The reference (cmtip) calls the third-party ``finufft`` library at
``cmtip/nufft/forward.py:40`` (``nufft3d2(H_, K_, L_, ugrid, out=, eps=1e-12,
isign=-1)``) and ``cmtip/nufft/adjoint.py:33`` (``nufft3d1(H_, K_, L_, nuvect,
out=, eps=1e-15, isign=1)``).  finufft is not vendored in the reference and is not
installed here (its version is unpinned in ``setup.py:11``), so this module
restates its published algorithm (Barnett, Magland & af Klinteberg, SIAM J. Sci.
Comput. 2019): ES-kernel spreading/interpolation (``oracle/nufft_ref.c``), an FFT of
the upsampled grid (numpy pocketfft) and deconvolution by the kernel's Fourier
transform (Gauss-Legendre quadrature).  ``nufft3d1``/``nufft3d2`` keep finufft's
Python call signatures so the module can stand in for ``finufft`` when the
reference itself is imported to generate golden fixtures.

Conventions (those of finufft's Python interface, which the reference relies on):
modes are centred, output index ``i`` along an axis holds mode ``k = i - M//2``;
array axis 0 pairs with the first coordinate array (H), axis 2 with the last (L).

``nudft3d1``/``nudft3d2`` are exact direct sums used to validate the fast oracle
("parity unpinned" against finufft itself: nothing of finufft runs here).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libcmt_oracle.so")
_lib = None


def build() -> str:
    """Compile the oracle's C restatement with its Makefile (gcc + OpenMP)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        lib = ctypes.CDLL(_LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        lib.cmto_spread.argtypes = [ctypes.c_int64, dp, dp, dp, dp, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_double, dp, ctypes.c_int]
        lib.cmto_interp.argtypes = [ctypes.c_int64, dp, dp, dp, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_double, dp, dp, ctypes.c_int]
        lib.cmto_max_threads.restype = ctypes.c_int
        _lib = lib
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def default_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:  # pragma: no cover
        return os.cpu_count() or 1


def es_params(eps: float, upsampfac: float = 2.0):
    """Kernel width w and shape beta for tolerance eps (ES-kernel paper, sec. 3)."""
    eps = max(float(eps), 1e-15)
    if upsampfac == 2.0:
        w = int(np.ceil(np.log10(1.0 / eps))) + 1
    else:
        w = int(np.ceil(np.log(1.0 / eps) / (np.pi * np.sqrt(1.0 - 1.0 / upsampfac))))
    w = max(2, min(w, 16))
    beta = 0.97 * np.pi * w * (1.0 - 0.5 / upsampfac)
    return w, float(beta)


def _nice(n: int) -> int:
    """Smallest even n' >= n whose only prime factors are 2, 3, 5."""
    m = max(n, 2)
    while True:
        if m % 2 == 0:
            r = m
            for p in (2, 3, 5):
                while r % p == 0:
                    r //= p
            if r == 1:
                return m
        m += 1


def fine_size(M: int, w: int, upsampfac: float = 2.0) -> int:
    return _nice(max(int(np.ceil(upsampfac * M)), 2 * w))


def kernel_ft(xi, w: int, beta: float, nquad: int = 128):
    """psi_hat(xi) = int_{-w/2}^{w/2} phi(t) cos(xi t) dt by Gauss-Legendre quadrature."""
    t, wt = np.polynomial.legendre.leggauss(nquad)
    t = 0.5 * w * 0.5 * (t + 1.0)          # nodes on [0, w/2]
    wt = 0.5 * w * 0.5 * wt
    z = 2.0 * t / w
    phi = np.exp(beta * (np.sqrt(np.maximum(1.0 - z * z, 0.0)) - 1.0))
    xi = np.asarray(xi, dtype=np.float64)
    return 2.0 * np.cos(np.multiply.outer(xi, t)) @ (wt * phi)


def modes(M: int):
    return np.arange(M) - M // 2


def _deconv(M, n, w, beta):
    k = modes(M)
    return 1.0 / kernel_ft(k * (2.0 * np.pi / n), w, beta)


def _as64(a):
    return np.ascontiguousarray(np.asarray(a).ravel(), dtype=np.float64)


def spread(x, y, z, c, n, w, beta, nthreads=None):
    lib = _load()
    x, y, z = _as64(x), _as64(y), _as64(z)
    c = np.ascontiguousarray(np.asarray(c).ravel(), dtype=np.complex128)
    grid = np.empty((n, n, n), dtype=np.complex128)
    lib.cmto_spread(x.size, _dp(x), _dp(y), _dp(z), _dp(c.view(np.float64)), n, w, beta,
                    _dp(grid.view(np.float64)), nthreads or default_threads())
    return grid


def interp(x, y, z, grid, w, beta, nthreads=None):
    lib = _load()
    x, y, z = _as64(x), _as64(y), _as64(z)
    grid = np.ascontiguousarray(grid, dtype=np.complex128)
    n = grid.shape[0]
    out = np.empty(x.size, dtype=np.complex128)
    lib.cmto_interp(x.size, _dp(x), _dp(y), _dp(z), n, w, beta, _dp(grid.view(np.float64)),
                    _dp(out.view(np.float64)), nthreads or default_threads())
    return out


def type1(x, y, z, c, M, eps=1e-12, isign=1, upsampfac=2.0, nthreads=None):
    """f_k = sum_j c_j exp(isign i k.x_j), k centred in [-M//2, (M-1)//2]^3, complex128."""
    w, beta = es_params(eps, upsampfac)
    n = fine_size(M, w, upsampfac)
    g = spread(x, y, z, c, n, w, beta, nthreads)
    G = np.fft.fftn(g) if isign < 0 else np.fft.ifftn(g) * float(n) ** 3
    idx = modes(M) % n
    p = _deconv(M, n, w, beta)
    f = G[np.ix_(idx, idx, idx)]
    return f * (p[:, None, None] * p[None, :, None] * p[None, None, :])


def type2(x, y, z, f, eps=1e-12, isign=-1, upsampfac=2.0, nthreads=None):
    """c_j = sum_k f_k exp(isign i k.x_j) for a cubic centred mode array f (M,M,M)."""
    f = np.asarray(f)
    M = f.shape[0]
    w, beta = es_params(eps, upsampfac)
    n = fine_size(M, w, upsampfac)
    p = _deconv(M, n, w, beta)
    G = np.zeros((n, n, n), dtype=np.complex128)
    idx = modes(M) % n
    G[np.ix_(idx, idx, idx)] = f * (p[:, None, None] * p[None, :, None] * p[None, None, :])
    g = np.fft.fftn(G) if isign < 0 else np.fft.ifftn(G) * float(n) ** 3
    return interp(x, y, z, g, w, beta, nthreads)


# --- finufft-compatible signatures (used when the reference is imported with stubs) ---

def nufft3d1(x, y, z, c, n_modes=None, out=None, eps=1e-6, isign=1, **kwargs):
    if out is not None:
        M = out.shape[0]
    else:
        M = n_modes[0] if hasattr(n_modes, "__len__") else int(n_modes)
    f = type1(x, y, z, c, M, eps=max(eps, 1e-14), isign=isign)
    if out is not None:
        out[...] = f.astype(out.dtype)
        return out
    return f


def nufft3d2(x, y, z, f, out=None, eps=1e-6, isign=-1, **kwargs):
    c = type2(x, y, z, f, eps=max(eps, 1e-14), isign=isign)
    if out is not None:
        out[...] = c.reshape(out.shape).astype(out.dtype)
        return out
    return c


# --- exact direct sums (small sizes) ---

def nudft3d1(x, y, z, c, M, isign=1, chunk=4096):
    k = modes(M).astype(np.float64)
    x, y, z = _as64(x), _as64(y), _as64(z)
    c = np.asarray(c).ravel().astype(np.complex128)
    f = np.zeros((M, M, M), dtype=np.complex128)
    for s in range(0, x.size, chunk):
        ex = np.exp(1j * isign * np.multiply.outer(x[s:s + chunk], k))
        ey = np.exp(1j * isign * np.multiply.outer(y[s:s + chunk], k))
        ez = np.exp(1j * isign * np.multiply.outer(z[s:s + chunk], k))
        f += np.einsum("j,ja,jb,jc->abc", c[s:s + chunk], ex, ey, ez, optimize=True)
    return f


def nudft3d2(x, y, z, f, isign=-1, chunk=4096):
    f = np.asarray(f).astype(np.complex128)
    M = f.shape[0]
    k = modes(M).astype(np.float64)
    x, y, z = _as64(x), _as64(y), _as64(z)
    out = np.empty(x.size, dtype=np.complex128)
    for s in range(0, x.size, chunk):
        ex = np.exp(1j * isign * np.multiply.outer(x[s:s + chunk], k))
        ey = np.exp(1j * isign * np.multiply.outer(y[s:s + chunk], k))
        ez = np.exp(1j * isign * np.multiply.outer(z[s:s + chunk], k))
        out[s:s + chunk] = np.einsum("abc,ja,jb,jc->j", f, ex, ey, ez, optimize=True)
    return out
