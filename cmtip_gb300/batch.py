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


class Instance:
    """One reconstruction of a batch: modes M, detector q-vectors ppr (3, n_pix) float64, the
    reciprocal extent, measured images (n_img, n_pix) and, when known, their orientations
    (n_img, 4) float32 quaternions."""

    def __init__(self, M, ppr, reciprocal_extent, images=None, orientations=None):
        self.M = int(M)
        self.ppr = torch.as_tensor(np.asarray(ppr, dtype=np.float64) if not torch.is_tensor(ppr) else ppr,
                                   dtype=torch.float64).reshape(3, -1)
        self.rext = float(reciprocal_extent)
        self.images = images
        self.orientations = orientations

    @property
    def n_pix(self):
        return self.ppr.shape[-1]


class BatchedReconstruction:
    """The stages of several independent reconstructions (cmtip's reconstruct loop,
    reconstruct.py:52-87, for many particles at once), one launch per NUFFT stage:

    * ``slices(acs, orientations)``: model slices Re(A_i ac_i) of every instance at the given
      orientations (align.py:39-65), one batched type-2 launch;
    * ``match(acs, n_ref)``: orientation matching of every instance's images against n_ref
      reference orientations (align.py:68-132): the references' slices of a group of
      instances in one batched launch (groups bounded by ``max_points``), then one
      persistent tensor-core distance launch over the group's instances and each
      instance's exact re-scoring;
    * ``solve(maxiter, estimates)``: every instance's autocorrelation solve
      (autocorrelation.py:176-248 with a fixed iteration count): the Toeplitz kernels (unit
      strengths onto 2M modes) in one batched launch, the right-hand sides (data onto M
      modes) in another, then every instance's CG iterations as the branches of one
      captured graph (``solve_many``).

    ``tuning``: None (defaults), "auto" (``tune.autotune`` per instance and transform), or a
    list of dicts (bin_size, maxsub) per instance.
    """

    def __init__(self, instances, eps=1e-6, prec=32, tuning=None, max_points=2_000_000_000, stream=None):
        self.inst = list(instances)
        self.eps, self.prec = float(eps), int(prec)
        self.tuning = tuning
        self.max_points = int(max_points)
        self.stream = stream
        self.stats = {}
        self._matchers = {}  # per instance: Matchers (per mode) and CG solvers, buffers kept across calls
        self._weights = {}

    # ---------------------------------------------------------------- helpers
    def _tuned(self, plan, i, kind, set_points, data):
        if self.tuning is None:
            if kind == "solve" and self.prec == 32:
                # solve_ac's Toeplitz workspace tuning: bins of 5 fine cells, 16384 points per
                # subproblem (the derived 2M plan then fits four CTAs per SM)
                return plan.set_tuning(5, 16384)
            return plan
        if self.tuning == "auto":
            from . import tune
            cfg = tune.autotune(plan.type, plan.M, set_points, data, prec=self.prec, eps=self.eps, isign=plan.isign,
                                tag=kind)
        else:
            cfg = self.tuning[i]
        return plan.set_tuning(int(cfg["bin_size"]), int(cfg["maxsub"]))

    def _timed(self, name, fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        out = fn()
        e1.record()
        torch.cuda.synchronize()
        self.stats[name] = self.stats.get(name, 0.0) + e0.elapsed_time(e1) / 1e3
        return out

    # ---------------------------------------------------------------- stages
    def _slice_group(self, idx, acs, quats, stat):
        """Batched type-2 slices of instances idx (acs, quats aligned with idx)."""
        from .nufft import inverse_rotations
        rt = torch.float64 if self.prec == 64 else torch.float32
        plans, modes = [], []
        for k, i in enumerate(idx):
            x = self.inst[i]
            inv, ppr = inverse_rotations(quats[k]), x.ppr.cuda()
            modes.append(torch.as_tensor(acs[k]).cuda().to(rt).reshape(-1))
            p = Plan(2, x.M, eps=self.eps, isign=-1, prec=self.prec)
            self._tuned(p, i, "slices", lambda pl, inv=inv, ppr=ppr, x=x: pl.set_pts_quat(inv, ppr, x.rext),
                        modes[-1])
            plans.append(p)

        def run():
            for k, i in enumerate(idx):
                x = self.inst[i]
                plans[k].set_pts_quat(inverse_rotations(quats[k]), x.ppr.cuda(), x.rext)
            b = Batch(plans, stream=self.stream)
            out = b.execute(modes, real_out=True)
            b.close()
            return out
        out = self._timed(stat, run)
        key = stat[:-2] + "_points"  # "<stage>_s" -> "<stage>_points"
        self.stats[key] = self.stats.get(key, 0) + sum(p.N for p in plans)
        for p in plans:
            p.close()
        return out

    def slices(self, acs, orientations=None):
        """Re(type-2 NUFFT of ac_i) at inv(R(q)) . ppr_i * pi / extent_i for every instance
        (orientations default to the instances' own); list of (n_i * n_pix_i,) tensors."""
        quats = orientations if orientations is not None else [x.orientations for x in self.inst]
        return self._slice_group(list(range(len(self.inst))), acs, quats, "slices_s")

    def _matcher(self, i, mode):
        from .alignment import Matcher, generate_weights
        key = (i, mode)
        if key not in self._matchers:
            x = self.inst[i]
            self._matchers[key] = Matcher(x.n_pix, mode)
            self._weights[i] = generate_weights(x.ppr.cpu().numpy().reshape(3, 1, -1), order=0)
        return self._matchers[key]

    def match(self, acs, n_ref, mode="bf16", ref_orientations=None):
        """Best reference orientation of every image of every instance: list of
        (quaternions (n_img, 4) float32 numpy, info dict).  Per group of instances: the
        references' slices in one batched interpolation launch, every instance's operands,
        then (tensor-core forms) ONE persistent distance launch over all the group's
        instances and one host synchronisation."""
        from .alignment import Matcher, reference_orientations
        refs = reference_orientations(n_ref, ref_orientations=ref_orientations)  # float32, as match_orientations
        results = [None] * len(self.inst)
        groups, cur, pts = [], [], 0
        for i in range(len(self.inst)):  # groups whose reference slices fit the point budget
            n = len(refs) * self.inst[i].n_pix
            if cur and pts + n > self.max_points:
                groups.append(cur)
                cur, pts = [], 0
            cur.append(i)
            pts += n
        if cur:
            groups.append(cur)
        grouped = mode in ("bf16", "bf16x3")
        for g in groups:
            matchers = [self._matcher(i, mode) for i in g]
            models = self._slice_group(g, [acs[i] for i in g], [refs] * len(g), "match_slices_s")

            def run(models=models, g=g, matchers=matchers):
                for k, i in enumerate(g):
                    x = self.inst[i]
                    matchers[k].set_data(torch.as_tensor(x.images).cuda().reshape(-1, x.n_pix), self._weights[i])
                    matchers[k].set_refs(models[k].reshape(len(refs), x.n_pix))
                if grouped:
                    if self.tuning == "auto":
                        from . import tune
                        tune.autotune_match(matchers)
                    return Matcher.run_many(matchers)
                return [mt.run() for mt in matchers]
            outs = self._timed("match_gemm_s", run)
            for k, i in enumerate(g):
                idx, d1, d2, tie, n_near = outs[k]
                index = idx.cpu().numpy().astype(np.int64)
                results[i] = (refs[index], dict(index=index, best=d1.cpu().numpy(), second=d2.cpu().numpy(),
                                                near_ties=int(n_near), refs=refs))
            del models
        return results

    def solve(self, maxiter=20, estimates=None, rtol=0.0, data=None, orientations=None):
        """Every instance's autocorrelation solve (solve_ac with a fixed iteration count and
        the instances' known orientations); list of float64 (M, M, M) tensors."""
        from .autocorrelation import TOEPLITZ, CGSolver, solve_many, support_from_estimate
        from .nufft import inverse_rotations
        K = len(self.inst)
        rt = torch.float64 if self.prec == 64 else torch.float32
        quats = orientations if orientations is not None else [x.orientations for x in self.inst]
        plans_M, plans_2M, solvers, sups, x0s, datas, rl = [], [], [], [], [], [], []
        for i, x in enumerate(self.inst):
            M, Mtot = x.M, x.M ** 3
            img = torch.as_tensor(data[i] if data is not None else x.images).cuda().reshape(-1)
            N = img.numel()
            p = Plan(1, M, eps=self.eps, isign=1, prec=self.prec)
            inv = inverse_rotations(quats[i])
            ppr = x.ppr.cuda()
            self._tuned(p, i, "solve", lambda pl, inv=inv, ppr=ppr, x=x: pl.set_pts_quat(inv, ppr, x.rext),
                        img.to(rt))
            plans_M.append(p)
            plans_2M.append(p.derive(1, 2 * M, isign=1))
            key = ("solver", i, self.prec)  # kept across calls: buffers and cuFFT plans
            if key not in self._matchers:
                self._matchers[key] = CGSolver(M, prec=self.prec, op=TOEPLITZ)
            solvers.append(self._matchers[key])
            if estimates is None or estimates[i] is None:
                sups.append(torch.ones(Mtot, dtype=torch.float32, device="cuda"))
                x0s.append(torch.zeros(Mtot, dtype=torch.float64, device="cuda"))
            else:
                est = torch.as_tensor(estimates[i]).cuda().to(torch.float32).contiguous()
                sups.append(support_from_estimate(est, inplace=True).reshape(-1))
                x0s.append(est.reshape(-1).to(torch.float64))
            datas.append(img.to(rt))
            rl.append(Mtot / N / 1000)

        def run():
            for p, x, q in zip(plans_M, self.inst, quats):
                p.set_pts_quat(inverse_rotations(q), x.ppr.cuda(), x.rext)
            b2 = Batch(plans_2M, stream=self.stream)
            kernels = b2.execute(None, real_out=True, fft_order=True,
                                 scale=[1.0 / float(2 * x.M) ** 3 for x in self.inst])
            bM = Batch(plans_M, stream=self.stream)
            adbs = bM.execute(datas, real_out=True, support=sups, scale=[1.0 / float(x.M) ** 3 for x in self.inst])
            ds, xs = [], []
            for i in range(K):
                solvers[i].set_operator(sups[i], 1.0, rl[i], 1e3)
                solvers[i].set_kernel(kernels[i])
                ds.append((adbs[i].reshape(-1).to(torch.float64) + rl[i] * x0s[i]).to(solvers[i].dtype).contiguous())
                xs.append(x0s[i].to(solvers[i].dtype).clone())
            # every instance's CG iterations as branches of one captured graph
            solve_many(solvers, ds, xs, maxiter=maxiter, rtol=rtol)
            b2.close()
            bM.close()
            return [x.to(torch.float64).reshape((inst.M,) * 3) for x, inst in zip(xs, self.inst)]
        out = self._timed("solve_s", run)
        self.stats["solve_points"] = 2 * sum(p.N for p in plans_M)
        for p in plans_2M + plans_M:
            p.close()
        return out
