"""Many independent reconstructions at once: batched NUFFT plans (``cmt_batch``).

A ``Batch`` holds plans of one type, precision, sign and kernel width, each with its own
modes M, points, tuning and fine grid.  ``execute`` runs every plan's grid preparation,
ONE persistent spreading (type 1) or interpolation (type 2) launch over the subproblems of
all plans -- its CTAs take (plan, bin, offset) work items from a device counter, so small
and large reconstructions share the GPU without a launch each -- then every plan's FFT and
deconvolution.  Results equal each plan's own ``Plan.execute`` up to floating-point
summation order.

The reference (cmtip) reconstructs one particle per process; this module has no
counterpart there.  ``BatchedReconstruction`` strings the stages of several
reconstructions together (slicing, orientation matching, autocorrelation solve) with one
launch per NUFFT stage.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .nufft import Plan, _cplx_dtype, _ptr, _real_dtype, _stream_ptr


class Batch:
    """Batched execution of ``plans`` (kept alive by the batch)."""

    def __init__(self, plans, stream=None):
        self.plans = list(plans)
        if not self.plans:
            raise ValueError("empty batch")
        p0 = self.plans[0]
        self.type, self.prec, self.device = p0.type, p0.prec, p0.device
        self.stream = stream if stream is not None else torch.cuda.current_stream(self.device)
        arr = (ctypes.c_void_p * len(self.plans))(*[p._h.value for p in self.plans])
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.call("cmt_batch_create", len(self.plans), arr, _stream_ptr(self.stream), ctypes.byref(h))
        self._h = h

    def profile(self, enable=True):
        _lib.call("cmt_batch_profile", self._h, int(bool(enable)))

    def last_ms(self):
        """(ms of the last batched kernel launch, work items) when profiling is on."""
        ms, nw = ctypes.c_float(), ctypes.c_int64()
        _lib.call("cmt_batch_last_ms", self._h, ctypes.byref(ms), ctypes.byref(nw))
        return ms.value, nw.value

    def execute(self, data, out=None, support=None, scale=None, real_out=False, fft_order=False):
        """data[i]: plan i's strengths (type 1; None = unit strengths for every plan) or modes
        (type 2).  Returns the list of outputs (M_i^3 modes or N_i values)."""
        K = len(self.plans)
        if data is None:
            data = [None] * K
        if len(data) != K:
            raise ValueError(f"expected {K} inputs")
        ones = data[0] is None
        if any((d is None) != ones for d in data):
            raise ValueError("unit strengths must be used by every plan of the batch or by none")
        if ones and self.type != 1:
            raise ValueError("only type 1 accepts implicit unit strengths")
        ins = []
        real_in = True
        if not ones:
            real_in = not data[0].is_complex()
            for p, d in zip(self.plans, data):
                d = d.to(p.device)
                if d.is_complex() == real_in:
                    raise ValueError("inputs must be all real or all complex")
                d = d.to(_real_dtype(p.prec) if real_in else _cplx_dtype(p.prec)).reshape(-1).contiguous()
                need = p.N if self.type == 1 else p.M ** 3
                if d.numel() != need:
                    raise ValueError(f"expected {need} input values, got {d.numel()}")
                ins.append(d)
        flags = (_lib.CMT_REAL_IN if real_in else 0) | (_lib.CMT_REAL_OUT if real_out else 0) | \
            (_lib.CMT_MODEORD_FFT if fft_order else 0)
        odt = _real_dtype(self.prec) if real_out else _cplx_dtype(self.prec)
        outs = []
        for i, p in enumerate(self.plans):
            shape = (p.M,) * 3 if self.type == 1 else (p.N,)
            o = out[i] if out is not None else torch.empty(shape, dtype=odt, device=p.device)
            if o.dtype != odt or o.numel() != int(np.prod(shape)) or not o.is_contiguous():
                raise ValueError(f"bad output tensor {i}")
            outs.append(o)
        sups = None
        keep = []
        if support is not None:
            keep = [torch.as_tensor(s_, device=p.device).to(torch.float32).contiguous()
                    for p, s_ in zip(self.plans, support)]
            sups = (ctypes.c_void_p * K)(*[t.data_ptr() for t in keep])
        scl = None if scale is None else (ctypes.c_double * K)(*[float(x) for x in scale])
        vals = (ctypes.c_void_p * K)(*[(0 if ones else ins[i].data_ptr()) if self.type == 1 else outs[i].data_ptr()
                                       for i in range(K)])
        modes = (ctypes.c_void_p * K)(*[outs[i].data_ptr() if self.type == 1 else ins[i].data_ptr()
                                        for i in range(K)])
        with torch.cuda.device(self.device):
            _lib.call("cmt_batch_execute", self._h, vals, modes, sups, scl, flags)
        self._keep = (ins, keep, outs)  # alive until the batch's stream has used them
        return outs

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.call("cmt_batch_destroy", self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
