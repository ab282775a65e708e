"""Orientation matching on the GPU, mirroring ``cmtip.alignment.align``.

``match_orientations`` keeps the reference's signature and behaviour
(``cmtip/alignment/align.py:68-132``): ``n_ref_orientations`` rounded up to a multiple of
``nbatches``; uniform reference quaternions (float32), optionally with the true
orientations spliced in and shuffled by numpy's global generator; per batch, model slices
by the type-2 NUFFT of the autocorrelation (real part) scaled by
``std(data) / std(batch)``; weighted euclidean distances; argmin over references
(first index on ties).  Keyword ``mode`` picks the distance form: ``"bf16"`` (tcgen05
tensor cores, TOPK candidates re-scored exactly), ``"fp32"`` or ``"fp64"`` (plain SIMT
forms).  ``return_info=True`` adds the near-tie count and distances.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .geometry import uniform_quaternions
from .nufft import DEFAULT_EPS, Plan, _ptr, _stream_ptr, get_plan, inverse_rotations

MODES = {"bf16": 0, "fp32": 1, "fp64": 2, "bf16x3": 3}


def generate_weights(pixel_position_reciprocal, order=0):
    """align.py:11-24: 1 / |s|^order with s in inverse Angstrom, normalised to sum 1 (float64)."""
    s = np.linalg.norm(np.asarray(pixel_position_reciprocal), axis=0) * 1e-10
    w = 1.0 / (s ** order)
    return w / np.sum(w)


def _ppr2d(pixel_position_reciprocal):
    p = pixel_position_reciprocal
    t = p if torch.is_tensor(p) else torch.from_numpy(np.ascontiguousarray(p, dtype=np.float64))
    return t.to("cuda", torch.float64).reshape(3, -1).contiguous()


def compute_slices(orientations, pixel_position_reciprocal, reciprocal_extent, ac, use_gpu=True,
                   eps=DEFAULT_EPS, prec=32, plan: Plan | None = None):
    """align.py:39-65: Re(type-2 NUFFT of ac) at inv(R(q)) . ppr * pi / reciprocal_extent,
    flattened (n_orientations * n_pix).  numpy in -> numpy out."""
    numpy_io = not torch.is_tensor(ac)
    acd = ac if torch.is_tensor(ac) else torch.from_numpy(np.ascontiguousarray(ac))
    acd = acd.to("cuda", torch.float64 if prec == 64 else torch.float32)
    M = acd.shape[0]
    if plan is None:
        plan = Plan(2, M, eps=eps, isign=-1, prec=prec)
    plan.set_pts_quat(inverse_rotations(orientations), _ppr2d(pixel_position_reciprocal), float(reciprocal_extent))
    out = plan.execute(acd.reshape(-1), real_out=True)
    return out.cpu().numpy() if numpy_io else out


class Matcher:
    """Device matcher (``cmt_match``): images fixed, references swappable."""

    def __init__(self, n_pix, mode="bf16", stream=None):
        self.mode = MODES[mode] if isinstance(mode, str) else int(mode)
        self.n_pix = int(n_pix)
        self.stream = stream if stream is not None else torch.cuda.current_stream()
        h = ctypes.c_void_p()
        _lib.call("cmt_match_create", self.n_pix, self.mode, _stream_ptr(self.stream), ctypes.byref(h))
        self._h = h
        self._keep = {}

    @property
    def dtype(self):
        return torch.float64 if self.mode == 2 else torch.float32

    def set_data(self, slices: torch.Tensor, weights):
        x = slices.to("cuda", self.dtype).reshape(-1, self.n_pix).contiguous()
        w = torch.as_tensor(np.asarray(weights, dtype=np.float64).reshape(-1) if not torch.is_tensor(weights)
                            else weights, device="cuda").to(torch.float64).contiguous()
        _lib.call("cmt_match_set_data", self._h, x.shape[0], _ptr(x), _ptr(w))
        self._keep["data"], self._keep["w"] = x, w
        self.n_img = x.shape[0]

    def set_refs(self, model: torch.Tensor, nbatches=1):
        m = model.to("cuda", self.dtype).reshape(-1, self.n_pix).contiguous()
        _lib.call("cmt_match_set_refs", self._h, m.shape[0], _ptr(m), int(nbatches))
        self._keep["model"] = m
        self.nbatches = int(nbatches)
        self.n_ref = m.shape[0]

    def run(self):
        n = self.n_img
        idx = torch.empty(n, dtype=torch.int32, device="cuda")
        d1 = torch.empty(n, dtype=torch.float64, device="cuda")
        d2 = torch.empty(n, dtype=torch.float64, device="cuda")
        tie = torch.empty(n, dtype=torch.int32, device="cuda")
        nn = ctypes.c_int()
        _lib.call("cmt_match_run", self._h, _ptr(idx), _ptr(d1), _ptr(d2), _ptr(tie), ctypes.byref(nn))
        return idx, d1, d2, tie, nn.value

    @staticmethod
    def run_many(matchers):
        """The tensor-core runs of several matchers (one instance each, modes bf16 / bf16x3) as
        one persistent launch (``cmt_match_run_many``) and one host synchronisation: a list of
        (best index, best distance, second distance, near-tie flags, near-tie count)."""
        n = len(matchers)
        outs = []
        for m in matchers:
            k = m.n_img
            outs.append((torch.empty(k, dtype=torch.int32, device="cuda"), torch.empty(k, dtype=torch.float64, device="cuda"),
                         torch.empty(k, dtype=torch.float64, device="cuda"), torch.empty(k, dtype=torch.int32, device="cuda")))
        arr = lambda xs: (ctypes.c_void_p * n)(*xs)
        nn = (ctypes.c_int * n)()
        _lib.call("cmt_match_run_many", n, arr([m._h.value for m in matchers]), arr([o[0].data_ptr() for o in outs]),
                  arr([o[1].data_ptr() for o in outs]), arr([o[2].data_ptr() for o in outs]),
                  arr([o[3].data_ptr() for o in outs]), nn)
        return [o + (int(nn[i]),) for i, o in enumerate(outs)]

    def set_tile(self, bn=256, stages=4):
        """Tile of the tensor-core distance kernel (references per tile, TMA ring stages)."""
        _lib.call("cmt_match_set_tile", self._h, int(bn), int(stages))
        self.tile = (int(bn), int(stages))

    def set_wait_limit(self, seconds):
        """Limit of the tensor-core pipeline's bounded waits (a run that exceeds it raises
        CmtError with code CMT_ERR_TIMEOUT; the matcher and the context stay usable)."""
        _lib.call("cmt_match_set_wait_limit", self._h, float(seconds))

    def profile(self, enable=True):
        _lib.call("cmt_match_profile", self._h, int(bool(enable)))

    def last_ms(self):
        """{set_data, set_refs, distance, rescore}: ms of the last calls (profile() on)."""
        ms = (ctypes.c_float * 4)()
        _lib.call("cmt_match_last_ms", self._h, ms)
        return dict(zip(("set_data", "set_refs", "distance", "rescore"), (float(v) for v in ms)))

    def stats(self):
        out = (ctypes.c_double * (self.nbatches + 1))()
        _lib.call("cmt_match_stats", self._h, out)
        return list(out)

    def close(self):
        if getattr(self, "_h", None):
            _lib.call("cmt_match_destroy", self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_MATCHERS = {}


def _matcher(n_pix, mode) -> "Matcher":
    """Matchers reused across calls with the same pixel count and form (operand buffers kept)."""
    key = (int(n_pix), mode, torch.cuda.current_device(), torch.cuda.current_stream().cuda_stream)
    mt = _MATCHERS.get(key)
    if mt is None:
        if len(_MATCHERS) >= 4:
            _MATCHERS.pop(next(iter(_MATCHERS))).close()
        mt = _MATCHERS[key] = Matcher(n_pix, mode=mode)
    return mt


def reference_orientations(n_ref_orientations, nbatches=1, true_orientations=None, ref_orientations=None):
    """align.py:96-111: n_ref rounded up to a multiple of nbatches; uniform quaternions as
    float32; true orientations spliced over the tail and the whole set shuffled."""
    quot, rem = divmod(n_ref_orientations, nbatches)
    if rem != 0:
        n_ref_orientations = (quot + 1) * nbatches
    refs = uniform_quaternions(n_ref_orientations) if ref_orientations is None else np.asarray(ref_orientations)
    refs = refs.astype(np.float32)
    if true_orientations is not None:
        refs = np.vstack((refs[:-len(true_orientations)], true_orientations))
        np.random.shuffle(refs)
    return refs


def match_orientations(generation, pixel_position_reciprocal, reciprocal_extent, slices_, ac, n_ref_orientations,
                       nbatches=1, order=0, use_gpu=True, true_orientations=None, *, ref_orientations=None,
                       mode="bf16", eps=DEFAULT_EPS, return_info=False):
    """align.py:68-132 on the GPU.  Returns the matched reference quaternions (float32, numpy)."""
    refs = reference_orientations(n_ref_orientations, nbatches, true_orientations, ref_orientations)
    n_ref = refs.shape[0]
    n_pix = int(np.asarray(pixel_position_reciprocal).shape[-1]) if not torch.is_tensor(pixel_position_reciprocal) \
        else int(pixel_position_reciprocal.shape[-1])
    prec = 64 if mode == "fp64" else 32
    acd = ac if torch.is_tensor(ac) else torch.from_numpy(np.ascontiguousarray(ac))
    acd = acd.to("cuda", torch.float64 if prec == 64 else torch.float32)
    plan = get_plan(2, acd.shape[0], eps=eps, isign=-1, prec=prec)  # cached: sort buffers reused
    model = compute_slices(refs, pixel_position_reciprocal, reciprocal_extent, acd, eps=eps, prec=prec, plan=plan)
    data = slices_ if torch.is_tensor(slices_) else torch.from_numpy(np.ascontiguousarray(slices_))
    data = data.to("cuda").reshape(-1, n_pix)
    weights = generate_weights(pixel_position_reciprocal if not torch.is_tensor(pixel_position_reciprocal)
                               else pixel_position_reciprocal.cpu().numpy(), order=order)
    mt = _matcher(n_pix, mode)
    mt.set_data(data, weights)
    mt.set_refs(model.reshape(n_ref, n_pix), nbatches=nbatches)
    idx, d1, d2, tie, n_near = mt.run()
    index = idx.cpu().numpy().astype(np.int64)
    for s in mt.stats()[:-1]:
        print(f"Data/Model std ratio: {s}.", flush=True)
    out = refs[index]
    if return_info:
        return out, dict(index=index, best=d1.cpu().numpy(), second=d2.cpu().numpy(),
                         near_ties=int(n_near), refs=refs)
    return out


def match_orientations_mult(generation, pixel_position_reciprocal, reciprocal_extent, slices_, ac_mult,
                            n_ref_orientations, nbatches=1, order=0, use_gpu=True, true_orientations=None, *,
                            ref_orientations=None, mode="bf16", eps=DEFAULT_EPS, return_info=False):
    """align.py:135-213 on the GPU: every image matched against each volume of ``ac_mult``
    (n_volumes, M, M, M), then assigned to the volume with the smallest best distance (first
    index on ties) and that volume's best reference.  The references are sorted once for all
    volumes and the images' operands built once; each volume costs one type-2 execute, one
    distance GEMM and one re-scoring.  Returns (quaternions float32 numpy, conformations
    int64 numpy)."""
    refs = reference_orientations(n_ref_orientations, nbatches, true_orientations, ref_orientations)
    n_ref = refs.shape[0]
    n_pix = int(np.asarray(pixel_position_reciprocal).shape[-1]) if not torch.is_tensor(pixel_position_reciprocal) \
        else int(pixel_position_reciprocal.shape[-1])
    prec = 64 if mode == "fp64" else 32
    rt = torch.float64 if prec == 64 else torch.float32
    vols = [a if torch.is_tensor(a) else torch.from_numpy(np.ascontiguousarray(a)) for a in ac_mult]
    M = vols[0].shape[0]
    plan = get_plan(2, M, eps=eps, isign=-1, prec=prec)
    plan.set_pts_quat(inverse_rotations(refs), _ppr2d(pixel_position_reciprocal), float(reciprocal_extent))
    data = slices_ if torch.is_tensor(slices_) else torch.from_numpy(np.ascontiguousarray(slices_))
    data = data.to("cuda").reshape(-1, n_pix)
    weights = generate_weights(pixel_position_reciprocal if not torch.is_tensor(pixel_position_reciprocal)
                               else pixel_position_reciprocal.cpu().numpy(), order=order)
    mt = _matcher(n_pix, mode)
    mt.set_data(data, weights)
    idx_all, best_all, near_all = [], [], []
    for v in vols:
        model = plan.execute(v.to("cuda", rt).reshape(-1), real_out=True)
        mt.set_refs(model.reshape(n_ref, n_pix), nbatches=nbatches)
        idx, d1, d2, tie, n_near = mt.run()
        for s in mt.stats()[:-1]:
            print(f"Data/Model std ratio: {s}.", flush=True)
        idx_all.append(idx.cpu().numpy().astype(np.int64))
        best_all.append(d1.cpu().numpy())
        near_all.append(int(n_near))
    best = np.stack(best_all)
    conformations = np.argmin(best, axis=0)
    index = np.stack(idx_all)[conformations, np.arange(best.shape[1])]
    out = refs[index], conformations
    if return_info:
        srt = np.sort(best, axis=0)
        # volumes whose best distances are within one FP32 rounding of each other
        vol_ties = int(np.sum(srt[1] - srt[0] <= srt[0] * 2.0 ** -23)) if best.shape[0] > 1 else 0
        return out + (dict(index=index, best=best, near_ties=near_all, volume_ties=vol_ties, refs=refs),)
    return out
