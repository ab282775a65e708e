"""Type-1 / type-2 NUFFT on the GPU, mirroring ``cmtip.nufft``.

``forward_gpu`` / ``adjoint_gpu`` keep the call signatures, argument meaning and error
behaviour of ``cmtip/nufft/forward.py:45-82`` and ``cmtip/nufft/adjoint.py:46-86``:

* forward: optional ``support`` multiplied into ``ugrid`` **in place** (forward.py:67-68),
  ``use_recip_sym`` keeps only ``ugrid.real`` (:69-70), type 2 with isign = -1, complex64
  output of the points' shape;
* adjoint: type 1 with isign = +1, ``* support``, ``.real`` if ``use_recip_sym``, ``/ M**3``;
* an ``AssertionError`` if any coordinate has ``|x| >= 3 pi`` (forward.py:64, adjoint.py:66).

Inputs may be numpy arrays (results come back as numpy, like the reference) or CUDA
torch tensors (results stay on the device).  ``Plan`` exposes the underlying plan
object for callers that reuse points across many transforms (the CG solver, the
alignment slicer).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib

DEFAULT_EPS = 1e-6

# When true, plans created afterwards record per-launch CUDA-event timings of their
# spread / interpolation kernels (read with Plan.profile_read); benchmarks use this.
PROFILE_KERNELS = False
_LIVE_PLANS = None  # weakref.WeakSet of plans created while PROFILE_KERNELS is set


def _stream_ptr(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _ptr(t: torch.Tensor):
    return ctypes.c_void_p(t.data_ptr())


def _real_dtype(prec):
    return torch.float64 if prec == 64 else torch.float32


def _cplx_dtype(prec):
    return torch.complex128 if prec == 64 else torch.complex64


class Plan:
    """A cubic 3D NUFFT plan (``cmt_plan``) bound to a CUDA stream.

    type 1: ``execute(c) -> f`` (N strengths to M^3 modes); type 2: ``execute(f) -> c``.
    """

    def __init__(self, nufft_type: int, M: int, eps: float = DEFAULT_EPS, isign: int | None = None,
                 prec: int = 32, upsampfac: float = 0.0, stream=None, device=None):
        self.type = int(nufft_type)
        self.M = int(M)
        self.prec = int(prec)
        self.isign = int(isign if isign is not None else (1 if self.type == 1 else -1))
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        with torch.cuda.device(self.device):
            self.stream = stream if stream is not None else torch.cuda.current_stream()
            h = ctypes.c_void_p()
            _lib.call("cmt_plan_create", self.type, self.M, self.prec, float(eps), self.isign,
                      float(upsampfac), _stream_ptr(self.stream), ctypes.byref(h))
        self._h = h
        self._src = None
        self.N = 0
        self._keep = ()
        if PROFILE_KERNELS:
            self.profile(True)
            global _LIVE_PLANS
            import weakref
            if _LIVE_PLANS is None:
                _LIVE_PLANS = weakref.WeakSet()
            _LIVE_PLANS.add(self)

    @property
    def N(self):
        return self._src.N if getattr(self, "_src", None) is not None else self._n

    @property
    def points_version(self) -> int:
        """Incremented whenever the plan's points (or its source plan's) are replaced."""
        src = getattr(self, "_src", None)
        return src.points_version if src is not None else getattr(self, "_pts_version", 0)

    def _bump_points(self):
        self._pts_version = getattr(self, "_pts_version", 0) + 1

    @N.setter
    def N(self, value):
        self._n = value

    def derive(self, nufft_type: int, M: int, isign: int | None = None) -> "Plan":
        """A plan on this plan's points with a fine grid twice as fine (no second sort):
        used for the Toeplitz kernel on 2M modes.  Keeps this plan alive."""
        d = Plan.__new__(Plan)
        d.type, d.M, d.prec = int(nufft_type), int(M), self.prec
        d.isign = int(isign if isign is not None else (1 if d.type == 1 else -1))
        d.device, d.stream = self.device, self.stream
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.call("cmt_plan_create_derived", self._h, d.type, d.M, d.isign, ctypes.byref(h))
        d._h, d._src, d._n, d._keep = h, self, 0, ()
        if PROFILE_KERNELS:
            d.profile(True)
            _LIVE_PLANS.add(d)
        return d

    # -- kernel timing
    def profile(self, enable=True):
        _lib.call("cmt_plan_profile", self._h, int(bool(enable)))

    def profile_read(self, max_launches=256):
        """[(ms, kind)] of the spread (kind 1) / interpolation (kind 2) launches since the last read."""
        ms = (ctypes.c_float * max_launches)()
        kinds = (ctypes.c_int * max_launches)()
        n = ctypes.c_int()
        _lib.call("cmt_plan_profile_read", self._h, ms, kinds, max_launches, ctypes.byref(n))
        return [(ms[i], kinds[i]) for i in range(n.value)]

    # -- info
    def info(self):
        n, w, bs = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        beta, nsub = ctypes.c_double(), ctypes.c_int64()
        _lib.call("cmt_plan_info", self._h, ctypes.byref(n), ctypes.byref(w), ctypes.byref(beta),
                  ctypes.byref(bs), ctypes.byref(nsub))
        return dict(n_fine=n.value, width=w.value, beta=beta.value, bin_size=bs.value, n_subproblems=nsub.value)

    # -- tuning (bin size, points per subproblem); drops the points
    def set_tuning(self, bin_size: int = 0, maxsub: int = 0) -> "Plan":
        _lib.call("cmt_plan_set_tuning", self._h, int(bin_size), int(maxsub))
        self.N = 0
        self._bump_points()
        return self

    def tuning(self) -> dict:
        bs, ms = ctypes.c_int(), ctypes.c_int()
        _lib.call("cmt_plan_get_tuning", self._h, ctypes.byref(bs), ctypes.byref(ms))
        return dict(bin_size=bs.value, maxsub=ms.value)

    # -- points
    def set_pts(self, x, y, z):
        dt = _real_dtype(self.prec)
        x, y, z = (torch.as_tensor(a, device=self.device).reshape(-1).to(dt).contiguous() for a in (x, y, z))
        if not (x.numel() == y.numel() == z.numel()):
            raise ValueError("coordinate arrays differ in length")
        with torch.cuda.device(self.device):
            _lib.call("cmt_set_pts", self._h, x.numel(), _ptr(x), _ptr(y), _ptr(z))
        self.N = x.numel()
        self._keep = (x, y, z)
        self._bump_points()
        return self

    def set_pts_quat(self, inv_rot: torch.Tensor, ppr: torch.Tensor, reciprocal_extent: float):
        """Points from inverse rotations (n_img, 3, 3) float64 and q-vectors (3, n_pix) float64."""
        inv_rot = inv_rot.to(self.device, torch.float64).contiguous()
        ppr = ppr.to(self.device, torch.float64).reshape(3, -1).contiguous()
        n_img, n_pix = inv_rot.shape[0], ppr.shape[1]
        with torch.cuda.device(self.device):
            _lib.call("cmt_set_pts_quat", self._h, n_img, _ptr(inv_rot), n_pix, _ptr(ppr), float(reciprocal_extent))
        self.N = n_img * n_pix
        self._keep = (inv_rot, ppr)
        self._bump_points()
        return self

    # -- execution
    def execute(self, data: torch.Tensor, out: torch.Tensor | None = None, support: torch.Tensor | None = None,
                scale: float = 1.0, real_out: bool = False, fft_order: bool = False):
        """type 1: data = N strengths (real or complex) -> M^3 modes; type 2: data = M^3 modes -> N values."""
        if self.N == 0:
            raise RuntimeError("set_pts must be called before execute")
        if data is None:
            # type 1 of unit strengths (no N-sized buffer)
            if self.type != 1:
                raise ValueError("only type 1 accepts implicit unit strengths")
            flags = _lib.CMT_REAL_IN | (_lib.CMT_REAL_OUT if real_out else 0) | \
                (_lib.CMT_MODEORD_FFT if fft_order else 0)
            odt = _real_dtype(self.prec) if real_out else _cplx_dtype(self.prec)
            out = out if out is not None else torch.empty((self.M,) * 3, dtype=odt, device=self.device)
            sup = None if support is None else torch.as_tensor(support, device=self.device).to(torch.float32).contiguous()
            with torch.cuda.device(self.device):
                _lib.call("cmt_execute", self._h, None, _ptr(out), _ptr(sup) if sup is not None else None,
                          float(scale), flags)
            return out
        data = data.to(self.device)
        real_in = not data.is_complex()
        data = data.to(_real_dtype(self.prec) if real_in else _cplx_dtype(self.prec)).contiguous()
        flags = (_lib.CMT_REAL_IN if real_in else 0) | (_lib.CMT_REAL_OUT if real_out else 0) | \
                (_lib.CMT_MODEORD_FFT if fft_order else 0)
        if self.type == 1:
            if data.numel() != self.N:
                raise ValueError(f"expected {self.N} strengths, got {data.numel()}")
            shape = (self.M,) * 3
        else:
            if data.numel() != self.M ** 3:
                raise ValueError(f"expected {self.M ** 3} modes, got {data.numel()}")
            shape = (self.N,)
        odt = _real_dtype(self.prec) if real_out else _cplx_dtype(self.prec)
        if out is None:
            out = torch.empty(shape, dtype=odt, device=self.device)
        elif out.dtype != odt or out.numel() != int(np.prod(shape)) or not out.is_contiguous():
            raise ValueError("bad output tensor")
        sup = None
        if support is not None:
            sup = torch.as_tensor(support, device=self.device).to(torch.float32).contiguous()
            if sup.numel() != self.M ** 3:
                raise ValueError("support must have M^3 elements")
        with torch.cuda.device(self.device):
            if self.type == 1:
                _lib.call("cmt_execute", self._h, _ptr(data), _ptr(out), _ptr(sup) if sup is not None else None,
                          float(scale), flags)
            else:
                _lib.call("cmt_execute", self._h, _ptr(out), _ptr(data), _ptr(sup) if sup is not None else None,
                          float(scale), flags)
        return out

    def execute_pair(self, f_in: torch.Tensor, out: torch.Tensor | None = None, support=None, scale: float = 1.0):
        """scale * S . Re(A^H A (S f_in)) on the plan's points (A: type 2 isign -1)."""
        dt = _real_dtype(self.prec)
        f_in = f_in.to(self.device, dt).contiguous()
        if out is None:
            out = torch.empty((self.M,) * 3, dtype=dt, device=self.device)
        sup = None if support is None else torch.as_tensor(support, device=self.device).to(torch.float32).contiguous()
        with torch.cuda.device(self.device):
            _lib.call("cmt_execute_pair", self._h, _ptr(f_in), _ptr(out), _ptr(sup) if sup is not None else None,
                      float(scale))
        return out

    def close(self):
        if getattr(self, "_h", None):
            _lib.call("cmt_plan_destroy", self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def inverse_rotations(quats, device=None) -> torch.Tensor:
    """``inv(quaternion2rot3d(q))`` for each float32 quaternion, on the device (n, 3, 3) float64."""
    q = torch.as_tensor(np.asarray(quats, dtype=np.float32) if not torch.is_tensor(quats) else quats)
    q = q.to(device or "cuda", torch.float32).reshape(-1, 4).contiguous()
    out = torch.empty((q.shape[0], 3, 3), dtype=torch.float64, device=q.device)
    with torch.cuda.device(q.device):
        _lib.call("cmt_inverse_rotations", _ptr(q), q.shape[0], _ptr(out), _stream_ptr())
    return out


# ------------------------------------------------------------ plan cache

_PLANS = {}


def get_plan(nufft_type, M, eps=DEFAULT_EPS, isign=None, prec=32, upsampfac=0.0) -> Plan:
    dev = torch.cuda.current_device()
    key = (nufft_type, M, eps, isign, prec, upsampfac, dev, torch.cuda.current_stream().cuda_stream)
    p = _PLANS.get(key)
    if p is None:
        if len(_PLANS) > 8:
            _PLANS.pop(next(iter(_PLANS))).close()
        p = Plan(nufft_type, M, eps=eps, isign=isign, prec=prec, upsampfac=upsampfac)
        _PLANS[key] = p
    return p


def clear_plan_cache():
    for p in _PLANS.values():
        p.close()
    _PLANS.clear()


# ------------------------------------------------------------ cmtip.nufft mirror

def _to_device(a, dtype=None):
    t = a if torch.is_tensor(a) else torch.from_numpy(np.ascontiguousarray(a))
    t = t.to("cuda")
    return t.to(dtype) if dtype is not None else t


def _check_range(H_, K_, L_):
    m = max(float(torch.as_tensor(a).abs().max()) if torch.is_tensor(a) else float(np.max(np.abs(a)))
            for a in (H_, K_, L_))
    assert m < 3 * np.pi


def forward_gpu(ugrid, H_, K_, L_, support=None, use_recip_sym=True, eps=DEFAULT_EPS, prec=32):
    """Type-2 NUFFT (isign -1) of ``ugrid`` at (H_, K_, L_); cmtip/nufft/forward.py:45-82."""
    numpy_io = not torch.is_tensor(ugrid)
    shape = tuple(np.shape(H_)) if not torch.is_tensor(H_) else tuple(H_.shape)
    if support is not None:
        ugrid *= support  # in place, as the reference does (forward.py:67-68)
    g = _to_device(ugrid)
    if use_recip_sym and g.is_complex():
        g = g.real
    M = g.shape[0]
    plan = get_plan(2, M, eps=eps, isign=-1, prec=prec)
    plan.set_pts(_to_device(H_), _to_device(K_), _to_device(L_))
    out = plan.execute(g.reshape(-1)).reshape(shape)
    if prec == 32:
        out = out.to(torch.complex64)
    return out.cpu().numpy() if numpy_io else out


def adjoint_gpu(nuvect, H_, K_, L_, M, use_recip_sym=True, support=None, eps=DEFAULT_EPS, prec=32):
    """Type-1 NUFFT (isign +1) onto M^3 modes, * support, .real, / M**3; cmtip/nufft/adjoint.py:46-86."""
    numpy_io = not torch.is_tensor(nuvect)
    c = _to_device(nuvect).reshape(-1)
    plan = get_plan(1, int(M), eps=eps, isign=1, prec=prec)
    plan.set_pts(_to_device(H_), _to_device(K_), _to_device(L_))
    sup = None if support is None else _to_device(support, torch.float32)
    out = plan.execute(c, support=sup, scale=1.0 / float(M) ** 3, real_out=bool(use_recip_sym))
    return out.cpu().numpy() if numpy_io else out


# the reference selects these by use_gpu; the CUDA path is the only implementation here
forward = forward_gpu
adjoint = adjoint_gpu
