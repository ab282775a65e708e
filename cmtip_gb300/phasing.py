"""Phase retrieval on the GPU, mirroring ``cmtip.phasing.phase``.

Same functions, arguments and in-place behaviour as the reference (cmtip/phasing/phase.py):
``ER`` / ``HIO`` / ``recenter`` overwrite ``rho_`` (and ``support_``), ``shrink_wrap``
overwrites ``support_``, ``phase`` returns ``(ac_phased, support_, rho_)`` with a caller's
``support_`` / ``rho_`` updated in place.  Arrays keep the reference's convention: a trailing
underscore means FFT order (DC term at the corner).  numpy arguments are copied to the GPU
and results copied back (numpy in, numpy out); CUDA tensors stay on the device and are
updated in place when they already have the working type.

Every operation runs in the CUDA kernels of ``csrc/phase.cu`` (cuFFT for the transforms);
an ER or HIO loop replays one captured graph per iteration.  The working precision follows
the density's dtype in the single-step functions (float64 -> the reference's double
arithmetic, float32 -> single) and the ``prec`` keyword in ``phase``: 32 by default, as the
rest of this library (the reference's 1300-iteration schedule at M = 81 in 0.036 s against
0.245 s for ``prec=64``; GB300's double-precision FFTs are slow), 64 for the reference's
arithmetic.  ER / HIO from a random start are chaotic, so the two forms follow different
trajectories from the first rounding difference and reach solutions of the same quality.
``phase`` draws its random initial density from numpy's global generator exactly as the
reference does (phase.py:200-201), so a seeded reference run and this one start alike.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .nufft import _ptr, _stream_ptr

DEFAULT_PREC = 32  # phase(); the single-step functions follow the density's dtype

_PHASERS: dict = {}


def _gauss_taps(sigma, truncate=2.0):
    """Normalised Gaussian taps of scipy.ndimage.gaussian_filter (radius = int(truncate *
    sigma + 0.5), weights exp(-x^2 / 2 sigma^2) / sum) as float64, and the radius."""
    radius = int(truncate * float(sigma) + 0.5)
    x = np.arange(-radius, radius + 1)
    phi = np.exp(-0.5 / (float(sigma) * float(sigma)) * x ** 2)
    return np.ascontiguousarray(phi / phi.sum(), dtype=np.float64), radius


class Phaser:
    """Device workspace for grids of edge M in one precision (``cmt_phaser``)."""

    def __init__(self, M, prec=DEFAULT_PREC, device=None, stream=None):
        self.M, self.prec = int(M), int(prec)
        if self.prec not in (32, 64):
            raise ValueError("prec must be 32 or 64")
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.dtype = torch.float64 if self.prec == 64 else torch.float32
        with torch.cuda.device(self.device):
            self.stream = stream if stream is not None else torch.cuda.current_stream()
            h = ctypes.c_void_p()
            _lib.call("cmt_phase_create", self.M, self.prec, _stream_ptr(self.stream), ctypes.byref(h))
        self._h = h

    def _call(self, name, *args):
        with torch.cuda.device(self.device):
            _lib.call(name, self._h, *args)

    def amplitudes(self, ac, sigma=1.0, truncate=2.0):
        """(ac_filt_, amplitudes_) of phase.py:186-192 from a centred autocorrelation."""
        M = self.M
        acd = ac.to(self.device, torch.float64).contiguous()
        w, r = _gauss_taps(sigma, truncate)
        ac_filt_ = torch.empty((M, M, M), dtype=torch.float64, device=self.device)
        amp = torch.empty((M, M, M), dtype=self.dtype, device=self.device)
        self._call("cmt_phase_amplitudes", _ptr(acd), w.ctypes.data_as(ctypes.c_void_p), r, _ptr(ac_filt_), _ptr(amp))
        return ac_filt_, amp

    def create_support(self, ac_filt_, mquat):
        sup = torch.empty((self.M,) * 3, dtype=torch.bool, device=self.device)
        self._call("cmt_phase_create_support", _ptr(ac_filt_), int(mquat), _ptr(sup))
        return sup

    def er(self, rho, amp, mask, sup, rho_max, n_loops):
        self._call("cmt_phase_er", _ptr(rho), _ptr(amp), _ptr(mask), _ptr(sup), float(rho_max), int(n_loops))

    def hio(self, beta, rho, amp, mask, sup, rho_max, n_loops):
        self._call("cmt_phase_hio", float(beta), _ptr(rho), _ptr(amp), _ptr(mask), _ptr(sup), float(rho_max),
                   int(n_loops))

    def step(self, rho, amp, mask, sup):
        rmod = torch.empty_like(rho)
        star = torch.empty(rho.shape, dtype=torch.bool, device=self.device)
        self._call("cmt_phase_step", _ptr(rho), _ptr(amp), _ptr(mask), _ptr(sup), _ptr(rmod), _ptr(star))
        return rmod, star

    def shrink_wrap(self, cutoff, sigma, rho, sup, truncate=2.0):
        w, r = _gauss_taps(sigma, truncate)
        self._call("cmt_phase_shrink_wrap", float(cutoff), w.ctypes.data_as(ctypes.c_void_p), r, _ptr(rho), _ptr(sup))

    def com_sums(self, rho, hkl=None):
        """(num[3], den) of center_of_mass as float64 numpy (one device-to-host read)."""
        sums = torch.empty(4, dtype=torch.float64, device=self.device)
        self._call("cmt_phase_center_of_mass", _ptr(rho), _ptr(hkl) if hkl is not None else None, _ptr(sums))
        s = sums.cpu().numpy()
        return s[:3], s[3]

    def roll(self, rho, sup, shifts):
        self._call("cmt_phase_roll", _ptr(rho) if rho is not None else None, _ptr(sup) if sup is not None else None,
                   *[int(s) for s in shifts])

    def autocorrelation(self, rho):
        out = torch.empty((self.M,) * 3, dtype=torch.float64, device=self.device)
        self._call("cmt_phase_autocorrelation", _ptr(rho), _ptr(out))
        return out

    def close(self):
        if getattr(self, "_h", None):
            _lib.call("cmt_phase_destroy", self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def get_phaser(M, prec=DEFAULT_PREC, device=None):
    """The cached Phaser for (device, M, prec, current stream)."""
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    with torch.cuda.device(dev):
        stream = torch.cuda.current_stream()
    key = (dev.index, int(M), int(prec), stream.cuda_stream)
    p = _PHASERS.get(key)
    if p is None:
        p = _PHASERS[key] = Phaser(M, prec, dev, stream)
    return p


# ---------------------------------------------------------------- argument plumbing

def _device_of(*arrays):
    for a in arrays:
        if torch.is_tensor(a) and a.is_cuda:
            return a.device
    return torch.device("cuda", torch.cuda.current_device())


def _as_tensor(a):
    if torch.is_tensor(a):
        return a
    return torch.from_numpy(np.ascontiguousarray(a))


class _Arg:
    """A caller's array as a contiguous device tensor of the working dtype; ``commit``
    writes a modified working copy back into the caller's array (numpy or tensor)."""

    def __init__(self, a, dtype, device):
        self.orig = a
        t = _as_tensor(a)
        if t.dtype == torch.bool and dtype == torch.uint8:
            t = t.to(device).contiguous()
            self.work = t.view(torch.uint8) if t.is_contiguous() else t.to(torch.uint8)
        elif dtype == torch.uint8:
            self.work = (t.to(device) != 0).to(torch.uint8).contiguous()
        else:
            self.work = t.to(device=device, dtype=dtype).contiguous()
        self.aliased = torch.is_tensor(a) and a.is_cuda and self.work.data_ptr() == a.data_ptr()

    def commit(self):
        if self.aliased:
            return
        src = self.work
        if torch.is_tensor(self.orig):
            if self.orig.dtype == torch.bool:
                src = src != 0
            self.orig.copy_(src.to(self.orig.device, self.orig.dtype).reshape(self.orig.shape))
        else:
            host = src.cpu().numpy()
            if self.orig.dtype == np.bool_:
                host = host != 0
            self.orig[...] = host.reshape(self.orig.shape)


def _prec_of(rho_):
    dt = rho_.dtype
    return 32 if dt in (np.float32, torch.float32) else 64


def _work_dtype(prec):
    return torch.float64 if prec == 64 else torch.float32


def _M_of(a):
    return int(a.shape[0])


# ---------------------------------------------------------------- reference functions

def center_of_mass(rho_, hkl_, M):
    """phase.py:11-23: np.round(sum(|rho_| hkl_) / sum(|rho_|) * M / 2), float64 numpy."""
    dev = _device_of(rho_, hkl_)
    prec = _prec_of(rho_)
    p = get_phaser(M, prec, dev)
    rho = _Arg(rho_, _work_dtype(prec), dev).work
    hkl = _as_tensor(hkl_).to(dev, torch.float64).contiguous()
    num, den = p.com_sums(rho, hkl)
    return np.round(num / den * M / 2)


def recenter(rho_, support_, M):
    """phase.py:26-44: roll rho_ and support_ so the centre of mass sits at the origin."""
    dev = _device_of(rho_, support_)
    prec = _prec_of(rho_)
    p = get_phaser(M, prec, dev)
    rho = _Arg(rho_, _work_dtype(prec), dev)
    sup = _Arg(support_, torch.uint8, dev)
    _recenter_device(p, rho.work, sup.work, M)
    rho.commit()
    sup.commit()


def _recenter_device(p, rho, sup, M):
    num, den = p.com_sums(rho)
    vect = np.round(num / den * M / 2)
    shifts = [int(vect[i]) for i in range(3)]  # int(nan) raises ValueError, as the reference
    p.roll(rho, sup, shifts)


def create_support_(ac_, M, Mquat, generation):
    """phase.py:47-64: centred cube of edge M - 2 Mquat (ifftshifted) and ac_ > 1e-2 max(ac_).
    numpy in -> numpy bool out; tensor in -> bool tensor on its device."""
    dev = _device_of(ac_)
    p = get_phaser(M, DEFAULT_PREC, dev)
    acf = _as_tensor(ac_).to(dev, torch.float64).contiguous()
    sup = p.create_support(acf, Mquat)
    return sup if torch.is_tensor(ac_) else sup.cpu().numpy()


def _loop_args(rho_, amplitudes_, amp_mask_, support_):
    dev = _device_of(rho_, amplitudes_, amp_mask_, support_)
    prec = _prec_of(rho_)
    dt = _work_dtype(prec)
    M = _M_of(rho_)
    p = get_phaser(M, prec, dev)
    return (p, _Arg(rho_, dt, dev), _Arg(amplitudes_, dt, dev).work, _Arg(amp_mask_, torch.uint8, dev).work,
            _Arg(support_, torch.uint8, dev).work)


def ER_loop(n_loops, rho_, amplitudes_, amp_mask_, support_, rho_max):
    """phase.py:67-72: n_loops ER iterations, rho_ in place."""
    p, rho, amp, mask, sup = _loop_args(rho_, amplitudes_, amp_mask_, support_)
    p.er(rho.work, amp, mask, sup, rho_max, n_loops)
    rho.commit()


def HIO_loop(n_loops, beta, rho_, amplitudes_, amp_mask_, support_, rho_max):
    """phase.py:75-80: n_loops HIO iterations, rho_ in place."""
    p, rho, amp, mask, sup = _loop_args(rho_, amplitudes_, amp_mask_, support_)
    p.hio(beta, rho.work, amp, mask, sup, rho_max, n_loops)
    rho.commit()


def ER(rho_, amplitudes_, amp_mask_, support_, rho_max):
    """phase.py:83-99: one Error Reduction step, rho_ in place."""
    ER_loop(1, rho_, amplitudes_, amp_mask_, support_, rho_max)


def HIO(beta, rho_, amplitudes_, amp_mask_, support_, rho_max):
    """phase.py:102-119: one Hybrid Input-Output step, rho_ in place."""
    HIO_loop(1, beta, rho_, amplitudes_, amp_mask_, support_, rho_max)


def step_phase(rho_, amplitudes_, amp_mask_, support_):
    """phase.py:122-144: (rho_mod_, support_star_)."""
    p, rho, amp, mask, sup = _loop_args(rho_, amplitudes_, amp_mask_, support_)
    rmod, star = p.step(rho.work, amp, mask, sup)
    if torch.is_tensor(rho_):
        return rmod, star
    return rmod.cpu().numpy(), star.cpu().numpy()


def shrink_wrap(cutoff, sigma, rho_, support_):
    """phase.py:147-162: support_ = gaussian_filter(|rho_|, sigma, 'wrap', truncate 2) >
    max|rho_| * cutoff, in place."""
    dev = _device_of(rho_, support_)
    prec = _prec_of(rho_)
    p = get_phaser(_M_of(rho_), prec, dev)
    rho = _Arg(rho_, _work_dtype(prec), dev).work
    sup = _Arg(support_, torch.uint8, dev)
    p.shrink_wrap(cutoff, sigma, rho, sup.work)
    sup.commit()


def phase(generation, ac, support_=None, rho_=None, n_iterations=10, nER=50, nHIO=25, prec=DEFAULT_PREC):
    """phase.py:165-219: n_iterations cycles of ER, HIO (beta 0.3), ER and shrink-wrap
    (cutoff 5e-2, sigma 1), a final ER loop, recentring, and the phased autocorrelation.

    Returns ``(ac_phased, support_, rho_)``: float64 centred autocorrelation, bool support
    and float64 density (FFT order).  numpy ``ac`` -> numpy results; a CUDA tensor ``ac``
    -> tensors on its device.  A caller's ``support_`` / ``rho_`` are updated in place and
    returned.  ``prec=64`` runs the reference's double arithmetic; the default ``prec=32``
    runs the iterations in single precision (a rounding-level change that the iteration,
    chaotic over many HIO steps, amplifies like any other)."""
    M = int(ac.shape[0])
    Mquat = int((M - 1) / 4)
    dev = _device_of(ac, support_, rho_)
    dt = _work_dtype(prec)
    p = get_phaser(M, prec, dev)
    ac_t = _as_tensor(ac)
    if ac_t.is_complex():
        ac_t = ac_t.real
    ac_filt_, amp = p.amplitudes(ac_t)
    mask = torch.ones((M, M, M), dtype=torch.uint8, device=dev)
    mask[0, 0, 0] = 0  # phase.py:194-195: the central peak keeps the density's own value

    if support_ is None:
        sup_arg = None
        sup = p.create_support(ac_filt_, Mquat).view(torch.uint8)
    else:
        sup_arg = _Arg(support_, torch.uint8, dev)
        sup = sup_arg.work
    if rho_ is None:
        # phase.py:200-201 with numpy's global generator, as the reference draws it
        s_host = (sup.cpu().numpy() != 0)
        rho_arg = None
        rho = torch.from_numpy(s_host * np.random.rand(*s_host.shape)).to(dev, dt)
    else:
        rho_arg = _Arg(rho_, dt, dev)
        rho = rho_arg.work

    rho_max = np.inf
    for _ in range(n_iterations):
        p.er(rho, amp, mask, sup, rho_max, nER)
        p.hio(0.3, rho, amp, mask, sup, rho_max, nHIO)
        p.er(rho, amp, mask, sup, rho_max, nER)
        p.shrink_wrap(5e-2, 1, rho, sup)
    p.er(rho, amp, mask, sup, rho_max, nER)
    _recenter_device(p, rho, sup, M)
    ac_phased = p.autocorrelation(rho)

    numpy_out = not torch.is_tensor(ac)
    if sup_arg is not None:
        sup_arg.commit()
        sup_out = support_
    else:
        sup_b = sup.view(torch.bool)
        sup_out = sup_b.cpu().numpy() if numpy_out else sup_b
    if rho_arg is not None:
        rho_arg.commit()
        rho_out = rho_
    else:
        rho64 = rho.to(torch.float64)
        rho_out = rho64.cpu().numpy() if numpy_out else rho64
    return (ac_phased.cpu().numpy() if numpy_out else ac_phased), sup_out, rho_out
