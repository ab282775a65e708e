"""Autocorrelation solve on the GPU, mirroring ``cmtip.autocorrelation.autocorrelation``.

``solve_ac`` keeps the reference's signature (``autocorrelation.py:176``) and behaviour:
support from ``gaussian_filter(ac_estimate, 0.5) > 1e-12`` with the estimate masked in
place (:217-220), ``alambda = 1``, ``rlambda = Mtot / N / 1000``, ``flambda = 1e3`` (:223-225),
CG from ``x0 = ac_estimate`` with scipy's stopping rule and ``maxiter = 100`` (:226, :239),
float64 ``(M, M, M)`` result of the real part (:240-243).  Extra keyword arguments select
the precision (``prec=32``: FP32 vectors and NUFFT, FP64 inner products and step scalars;
``prec=64``: the plain-FP64 GPU form), the data-term operator (``"toeplitz"`` as the
reference, or ``"pair"``: the fused type-2 then type-1 NUFFT pair) and the NUFFT tolerance.

``setup_linops`` returns ``(W, d)`` like the reference (:113-173); ``W`` is a scipy
``LinearOperator`` whose matvec runs on the GPU (numpy in, numpy out) and which also
exposes ``W.solver`` for device-resident use.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .nufft import DEFAULT_EPS, Plan, _ptr, _stream_ptr, inverse_rotations

TOEPLITZ, PAIR = 0, 1


def gen_F_antisupport(M):
    """autocorrelation.py:66-85: ones where |q| > pi on linspace(-pi, pi, M)^3 (|q| to 4 dp)."""
    lu = np.linspace(-np.pi, np.pi, M)
    q2 = lu[:, None, None] ** 2 + lu[None, :, None] ** 2 + lu[None, None, :] ** 2
    return np.around(np.sqrt(q2), 4) > np.pi


def gen_nonuniform_positions(orientations, pixel_position_reciprocal, device="cuda"):
    """autocorrelation.py:12-29 on the device: H, K, L = inv(R(q)) . ppr, float64 tensors of
    shape (n_images, n_panels, n_pixels)."""
    ppr = torch.as_tensor(np.asarray(pixel_position_reciprocal), device=device, dtype=torch.float64)
    q = np.asarray(orientations)
    if q.shape[0] > 0:
        rot = inverse_rotations(q.astype(np.float32) if q.dtype != np.float32 else q, device=device)
    else:
        rot = torch.eye(3, dtype=torch.float64, device=device)[None]
    hkl = torch.einsum("ijk,klm->jilm", rot, ppr)
    return hkl[0], hkl[1], hkl[2]


_MASKS = {}


def default_mask_fft(M, device):
    """ifftshift(gen_F_antisupport(M)) as float32 on the device, built once per (M, device):
    it depends on M only and takes tens of milliseconds of host work at M ~ 100."""
    key = (int(M), str(torch.device(device)))
    mask = _MASKS.get(key)
    if mask is None:
        if len(_MASKS) >= 32:
            _MASKS.pop(next(iter(_MASKS)))
        m = np.asarray(np.fft.ifftshift(gen_F_antisupport(int(M))), dtype=np.float32)
        mask = _MASKS[key] = torch.from_numpy(m).to(device).contiguous()
    return mask


class CGSolver:
    """Device CG solver of the reference's normal equations (``cmt_cg``)."""

    def __init__(self, M, prec=32, op=TOEPLITZ, stream=None, device=None):
        self.M, self.prec, self.op = int(M), int(prec), int(op)
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.dtype = torch.float64 if self.prec == 64 else torch.float32
        with torch.cuda.device(self.device):
            self.stream = stream if stream is not None else torch.cuda.current_stream()
            h = ctypes.c_void_p()
            _lib.call("cmt_cg_create", self.M, self.prec, self.op, _stream_ptr(self.stream), ctypes.byref(h))
        self._h = h
        self._keep = {}

    def set_kernel(self, t_circ: torch.Tensor):
        t = t_circ.to(self.device, self.dtype).contiguous()
        with torch.cuda.device(self.device):
            _lib.call("cmt_cg_set_kernel", self._h, _ptr(t))
        self._keep["kernel"] = t

    def set_operator(self, support, alambda, rlambda, flambda, mask_fft=None):
        sup = torch.as_tensor(support, device=self.device).to(torch.float32).contiguous()
        if mask_fft is None:
            mask = default_mask_fft(self.M, self.device)
        else:
            mask = torch.as_tensor(np.asarray(mask_fft, dtype=np.float32), device=self.device).contiguous()
        with torch.cuda.device(self.device):
            _lib.call("cmt_cg_set_operator", self._h, _ptr(mask), _ptr(sup), float(alambda), float(rlambda),
                      float(flambda))
        self._keep["support"], self._keep["mask"] = sup, mask

    def set_pair_plan(self, plan: Plan):
        with torch.cuda.device(self.device):
            _lib.call("cmt_cg_set_pair_plan", self._h, plan._h)
        self._keep["plan"] = plan

    def matvec(self, x: torch.Tensor, out: torch.Tensor | None = None):
        x = x.to(self.device, self.dtype).reshape(-1).contiguous()
        out = out if out is not None else torch.empty_like(x)
        with torch.cuda.device(self.device):
            _lib.call("cmt_cg_matvec", self._h, _ptr(x), _ptr(out))
        return out

    def solve(self, d, x0, maxiter=100, rtol=1e-5, atol=0.0, use_graph=True):
        d = d.to(self.device, self.dtype).reshape(-1).contiguous()
        x = x0.to(self.device, self.dtype).reshape(-1).clone()
        it, rho = ctypes.c_int(), ctypes.c_double()
        with torch.cuda.device(self.device):
            _lib.call("cmt_cg_solve", self._h, _ptr(d), _ptr(x), int(maxiter), float(rtol), float(atol),
                      int(bool(use_graph)), ctypes.byref(it), ctypes.byref(rho))
        return x, it.value

    def close(self):
        if getattr(self, "_h", None):
            _lib.call("cmt_cg_destroy", self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def support_from_estimate(ac_estimate: torch.Tensor, inplace: bool = True):
    """(gaussian_filter(est, 0.5) > 1e-12) as float32, est *= support (autocorrelation.py:217-220)."""
    est = ac_estimate
    M = est.shape[0]
    sup = torch.empty_like(est)
    scratch = torch.empty(2 * est.numel(), dtype=torch.float32, device=est.device)
    with torch.cuda.device(est.device):
        _lib.call("cmt_support_from_estimate", _ptr(est), M, _ptr(sup), _ptr(scratch), int(inplace), _stream_ptr())
    return sup


def toeplitz_kernel(plan_2M: Plan, M: int) -> torch.Tensor:
    """Re(type-1 of ones onto 2M modes) / (2M)^3 in FFT order (autocorrelation.py:141-148)."""
    M2 = 2 * M
    return plan_2M.execute(None, scale=1.0 / float(M2) ** 3, real_out=True, fft_order=True)


class _DeviceOperator:
    """scipy-compatible W (numpy matvec) backed by a CGSolver."""

    def __new__(cls, solver: CGSolver):
        from scipy.sparse.linalg import LinearOperator
        n = solver.M ** 3

        def mv(u):
            u = np.asarray(u)
            if np.iscomplexobj(u):
                u = u.real
            y = solver.matvec(torch.from_numpy(np.ascontiguousarray(u)))
            return y.cpu().numpy().astype(np.float64)

        op = LinearOperator(dtype=np.complex64, shape=(n, n), matvec=mv)
        op.solver = solver
        return op


def _as_device(a, dtype, device="cuda"):
    t = a if torch.is_tensor(a) else torch.from_numpy(np.ascontiguousarray(a))
    return t.to(device=device, dtype=dtype)


_COPY_STREAMS = {}


def _copy_stream(device):
    """One side stream per device for host-to-device copies: the caching allocator reuses a
    freed block only on the stream that allocated it, so a fresh stream per call would
    allocate the (multi-GB) destination anew every time."""
    key = torch.device(device).index
    s = _COPY_STREAMS.get(key)
    if s is None:
        s = _COPY_STREAMS[key] = torch.cuda.Stream(device=device)
    return s


def _as_device_async(a, dtype):
    """(device tensor, event): a host tensor in pinned memory is copied on a side stream so
    the copy overlaps the device work issued before the event is waited on; anything else
    is converted on the current stream (event None)."""
    if torch.is_tensor(a) and not a.is_cuda and a.is_pinned() and a.dtype == dtype and a.is_contiguous():
        main = torch.cuda.current_stream()
        side = _copy_stream(main.device)
        side.wait_stream(main)
        with torch.cuda.stream(side):
            t = torch.empty(a.shape, dtype=dtype, device="cuda")
            t.copy_(a, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(side)
        t.record_stream(main)
        return t, ev
    return _as_device(a, dtype), None


def setup_linops(H, K, L, data, ac_support, weights, x0, M, Mtot, N, reciprocal_extent,
                 alambda, rlambda, flambda, use_gpu=True, use_recip_sym=True, prec=32,
                 operator="toeplitz", eps=DEFAULT_EPS):
    """autocorrelation.py:113-173 on the GPU: returns (W, d) with d as float64 numpy (or a
    device tensor when ``data`` is a CUDA tensor)."""
    if not use_recip_sym:
        raise NotImplementedError("the GPU solver implements the reference's use_recip_sym=True path")
    numpy_io = not torch.is_tensor(data)
    dev = torch.device("cuda", torch.cuda.current_device())
    rt = torch.float64 if prec == 64 else torch.float32
    # H_ = H.flatten() / reciprocal_extent * pi (float64 when reciprocal_extent is a numpy float)
    xs = [(_as_device(a, torch.float64).reshape(-1) / float(reciprocal_extent) * np.pi).to(rt) for a in (H, K, L)]
    op = PAIR if operator == "pair" else TOEPLITZ
    solver = CGSolver(M, prec=prec, op=op)
    sup = _as_device(ac_support, torch.float32).reshape(-1)
    solver.set_operator(sup, alambda, rlambda, flambda)
    plan_M = Plan(1, M, eps=eps, isign=1, prec=prec).set_pts(*xs)
    if op == TOEPLITZ:
        plan_2M = plan_M.derive(1, 2 * M, isign=1)
        solver.set_kernel(toeplitz_kernel(plan_2M, M))
        plan_2M.close()
    else:
        solver.set_pair_plan(plan_M)
    db = _as_device(data, torch.float32).reshape(-1) * _as_device(weights, torch.float32).reshape(-1)
    adb = plan_M.execute(db.to(rt), support=sup, scale=1.0 / float(M) ** 3, real_out=True).reshape(-1)
    d = float(alambda) * adb.to(torch.float64) + float(rlambda) * _as_device(x0, torch.float64).reshape(-1)
    W = _DeviceOperator(solver)
    W.plan_M = plan_M
    return W, (d.cpu().numpy() if numpy_io else d)


class _Workspace:
    """Plans and solvers reused across solve_ac calls with the same (M, prec, operator, eps):
    the sorted-point buffers, fine grids and cuFFT plans are allocated once; one CG solver
    per CG precision shares the plans."""

    def __init__(self, M, prec, op, eps):
        self.M, self.op = int(M), int(op)
        self.solvers = {int(prec): CGSolver(M, prec=prec, op=op)}
        self.solver = self.solvers[int(prec)]
        self.plan_M = Plan(1, M, eps=eps, isign=1, prec=prec)
        if op == TOEPLITZ and prec == 32:
            # bins of 5 fine cells and 16384 points per subproblem: the derived 2M plan's bins
            # (10 cells) keep its shared-memory subgrid small; measured at 5000 images x 262144
            # pixels, M = 81: a solve_ac step of 160.6 ms against 166.3 ms with the defaults
            self.plan_M.set_tuning(5, 16384)
        # the 2M-mode plan borrows plan_M's sorted points (fine grid exactly twice as fine)
        self.plan_2M = self.plan_M.derive(1, 2 * M, isign=1) if op == TOEPLITZ else None

    def plans(self):
        return [p for p in (self.plan_M, self.plan_2M) if p is not None]

    def sweep_solvers(self, cg_prec, n):
        key = ("sweep", int(cg_prec))
        lst = self.solvers.get(key, [])
        while len(lst) < n:
            lst.append(CGSolver(self.M, prec=cg_prec, op=self.op))
        self.solvers[key] = lst
        return lst[:n]

    def cg_solver(self, cg_prec):
        s = self.solvers.get(int(cg_prec))
        if s is None:
            s = self.solvers[int(cg_prec)] = CGSolver(self.M, prec=cg_prec, op=self.op)
        return s


_WORKSPACES = {}


def _workspace(M, prec, op, eps, dev) -> _Workspace:
    key = (int(M), int(prec), int(op), float(eps), str(dev), torch.cuda.current_stream().cuda_stream)
    ws = _WORKSPACES.get(key)
    if ws is None:
        if len(_WORKSPACES) >= 4:
            _WORKSPACES.pop(next(iter(_WORKSPACES)))
        ws = _WORKSPACES[key] = _Workspace(M, prec, op, eps)
    return ws


def clear_workspaces():
    _WORKSPACES.clear()


def _support_and_x0(ac_estimate, Mtot, dev):
    """autocorrelation.py:213-220: the support (all ones without an estimate, else
    gaussian_filter(est, 0.5) > 1e-12) and x0 = the estimate masked by it (zeros without
    one); a float32 numpy estimate is masked in place, as the reference does."""
    if ac_estimate is None:
        return (torch.ones(Mtot, dtype=torch.float32, device=dev),
                torch.zeros(Mtot, dtype=torch.float64, device=dev))
    if torch.is_tensor(ac_estimate):
        est = ac_estimate.to(dev, torch.float32).contiguous()
    else:
        est = torch.from_numpy(np.ascontiguousarray(ac_estimate, dtype=np.float32)).to(dev)
    sup = support_from_estimate(est, inplace=True).reshape(-1)
    if isinstance(ac_estimate, np.ndarray) and ac_estimate.dtype == np.float32:
        ac_estimate *= sup.reshape(ac_estimate.shape).cpu().numpy()  # the reference masks in place
    return sup, est.reshape(-1).to(torch.float64)


def sweep_lambdas(Mtot, N, n):
    """(rlambda, flambda) of ranks 0 .. n-1 of the reference's lambda scan on n MPI ranks
    (cmtip/autocorrelation/autocorrelation_mpi.py:139-141): rlambda = Mtot / N * 2^(r - n/2),
    flambda = 1e5 * 10^(r - n//2), with N the number of data points one rank holds."""
    rl = [float(Mtot / np.int64(N) * 2 ** (r - n / 2)) for r in range(n)]
    fl = [1e5 * pow(10, r - n // 2) for r in range(n)]
    return np.array(rl), np.array(fl, dtype=np.float64)


def sweep_select(generation, rlambdas, v1s, v2s):
    """Index of the kept solution (autocorrelation_mpi.py:157-178): in generation 0 the
    largest rlambda among the solutions with ||x|| >= mean ||x||, later the corner of the
    L-curve, argmin(||x|| + ||W x - d||)."""
    rlambdas, v1s, v2s = (np.asarray(a, dtype=np.float64) for a in (rlambdas, v1s, v2s))
    if generation == 0:
        idx = v1s >= np.mean(v1s)
        imax = np.argmax(rlambdas[idx])
        return int(np.arange(len(v1s), dtype=int)[idx][imax])
    return int(np.argmin(v1s + v2s))


def solve_ac(generation, pixel_position_reciprocal, reciprocal_extent, slices_, M, orientations=None,
             ac_estimate=None, use_gpu=True, use_recip_sym=True, *, maxiter=100, rtol=1e-5, prec=32,
             operator="toeplitz", eps=DEFAULT_EPS, use_graph=True, return_info=False, rng=None, verbose=True,
             cg_prec=None):
    """autocorrelation.py:176-248 on the GPU.  Returns the float64 (M, M, M) autocorrelation
    (numpy for numpy inputs, a CUDA tensor for tensor inputs); with ``return_info`` also a
    dict with the iteration count.

    ``prec`` sets the NUFFT precision and, unless ``cg_prec`` is given, the CG's (32: FP32
    vectors and FFT convolutions with FP64 dot products, norms and step scalars; 64: all
    FP64).  ``cg_prec=64`` with ``prec=32`` is the reference's own precision split: FP32
    NUFFT (finufft single precision, cmtip/nufft/adjoint.py:32-33) and a complex128-accurate
    CG (scipy's cg on float64 d, :239)."""
    if not use_recip_sym:
        raise NotImplementedError("the GPU solver implements the reference's use_recip_sym=True path")
    numpy_io = not torch.is_tensor(slices_)
    dev = torch.device("cuda", torch.cuda.current_device())
    Mtot = M ** 3
    n_images = slices_.shape[0]
    N = int(np.prod(slices_.shape))
    if orientations is None:
        from .geometry import random_quaternions
        orientations = random_quaternions(n_images, rng or np.random.default_rng())
    rt = torch.float64 if prec == 64 else torch.float32
    ppr = _as_device(pixel_position_reciprocal, torch.float64).reshape(3, -1)
    quats = orientations if torch.is_tensor(orientations) else np.asarray(orientations, dtype=np.float32)
    inv_rot = inverse_rotations(quats, device=dev)
    sup, x0 = _support_and_x0(ac_estimate, Mtot, dev)
    alambda, rlambda, flambda = 1.0, Mtot / N / 1000, 1e3
    op = PAIR if operator == "pair" else TOEPLITZ
    if cg_prec not in (None, prec) and op == PAIR:
        raise ValueError("the pair operator runs in the NUFFT's precision (cg_prec must equal prec)")
    ws = _workspace(M, prec, op, eps, dev)
    solver, plan_M, plan_2M = ws.cg_solver(cg_prec or prec), ws.plan_M, ws.plan_2M
    solver.set_operator(sup, alambda, rlambda, flambda)
    # the intensities are first needed by the right-hand side, after the point sort and the
    # Toeplitz kernel: from pinned host memory their copy overlaps that work.  It is issued
    # after the small host-to-device copies above, which would otherwise wait behind it on
    # the copy engine and hold up the sort.
    data, data_ready = _as_device_async(slices_, torch.float32)
    data = data.reshape(-1)
    plan_M.set_pts_quat(inv_rot, ppr, float(reciprocal_extent))
    if op == TOEPLITZ:
        solver.set_kernel(toeplitz_kernel(plan_2M, M))
    else:
        solver.set_pair_plan(plan_M)
    if data_ready is not None:
        torch.cuda.current_stream().wait_event(data_ready)
    adb = plan_M.execute(data if data.dtype == rt else data.to(rt), support=sup, scale=1.0 / float(M) ** 3,
                         real_out=True).reshape(-1)
    d = alambda * adb.to(torch.float64) + rlambda * x0
    x, iters = solver.solve(d, x0, maxiter=maxiter, rtol=rtol, use_graph=use_graph)
    ac = x.to(torch.float64).reshape((M,) * 3)
    if verbose:
        print(f"Recovered AC in {iters} iterations.", flush=True)
    out = ac.cpu().numpy() if numpy_io else ac
    if return_info:
        return out, {"iterations": iters, "d": d, "x0": x0, "solver": solver}
    return out


def solve_ac_sweep(generation, pixel_position_reciprocal, reciprocal_extent, slices_, M, orientations=None,
                   ac_estimate=None, use_gpu=True, use_recip_sym=True, *, n_lambdas=8, maxiter=100, rtol=1e-5,
                   prec=32, cg_prec=64, eps=DEFAULT_EPS, return_info=False, rng=None, verbose=True):
    """The lambda scan of cmtip/autocorrelation/autocorrelation_mpi.py:99-190 (solve_ac_mpi)
    on one GPU: the n_lambdas ranks' solves share the points, the Toeplitz kernel and the
    type-1 of the data, and differ in (rlambda, flambda) (sweep_lambdas) and thus in
    d = A^H b + rlambda x0; their CG iterations run together as independent branches of one
    captured graph (cmt_cg_solve_many), each with scipy's stopping rule (rtol 1e-5,
    maxiter 100, autocorrelation_mpi.py:142,153).  The kept solution follows the
    reference's rule (sweep_select) on v1 = ||x||, v2 = ||W x - d||.  Every rank here holds
    the whole image set (N = all data points, as one rank of the reference holding all
    images).  The CG runs in double precision by default (``cg_prec=64``, the reference's
    complex128 cg): the scan's largest flambda, 1e5 * 10^(n/2), puts W's condition beyond
    what single-precision CG vectors resolve, and the L-curve pick then follows rounding
    (``cg_prec=32`` is available for the small-flambda ranks' speed).  Returns the kept
    float64 (M, M, M) autocorrelation; with ``return_info`` also the lambdas, v1, v2,
    iteration counts, all solutions and the kept index."""
    if not use_recip_sym:
        raise NotImplementedError("the GPU solver implements the reference's use_recip_sym=True path")
    numpy_io = not torch.is_tensor(slices_)
    dev = torch.device("cuda", torch.cuda.current_device())
    Mtot = M ** 3
    N = int(np.prod(slices_.shape))
    if orientations is None:
        from .geometry import random_quaternions
        orientations = random_quaternions(slices_.shape[0], rng or np.random.default_rng())
    rt = torch.float64 if prec == 64 else torch.float32
    ppr = _as_device(pixel_position_reciprocal, torch.float64).reshape(3, -1)
    quats = orientations if torch.is_tensor(orientations) else np.asarray(orientations, dtype=np.float32)
    inv_rot = inverse_rotations(quats, device=dev)
    sup, x0 = _support_and_x0(ac_estimate, Mtot, dev)
    rls, fls = sweep_lambdas(Mtot, N, n_lambdas)
    ws = _workspace(M, prec, TOEPLITZ, eps, dev)
    solvers = ws.sweep_solvers(cg_prec or prec, n_lambdas)
    data, data_ready = _as_device_async(slices_, torch.float32)
    ws.plan_M.set_pts_quat(inv_rot, ppr, float(reciprocal_extent))
    kern = toeplitz_kernel(ws.plan_2M, M)
    if data_ready is not None:
        torch.cuda.current_stream().wait_event(data_ready)
    data = data.reshape(-1)
    adb = ws.plan_M.execute(data if data.dtype == rt else data.to(rt), support=sup, scale=1.0 / float(M) ** 3,
                            real_out=True).reshape(-1).to(torch.float64)
    ds, xs = [], []
    for s, rl, fl in zip(solvers, rls, fls):
        s.set_operator(sup, 1.0, rl, fl)
        s.set_kernel(kern)
        ds.append((adb + rl * x0).to(s.dtype).contiguous())
        xs.append(x0.to(s.dtype).clone())
    its = solve_many(solvers, ds, xs, maxiter=maxiter, rtol=rtol)
    v1 = np.array([float(torch.linalg.norm(x.double())) for x in xs])
    # v2 = ||W x - d|| in double precision, as the reference's complex128 W * ret - d: with
    # flambda up to 1e5 * 10^(n/2) a single-precision matvec's rounding would swamp the residual
    check = ws.cg_solver(64)
    check.set_kernel(kern)
    v2 = []
    for x, rl, fl in zip(xs, rls, fls):
        check.set_operator(sup, 1.0, rl, fl)
        v2.append(float(torch.linalg.norm(check.matvec(x.double()) - (adb + rl * x0))))
    v2 = np.array(v2)
    keep = sweep_select(generation, rls, v1, v2)
    ac = xs[keep].to(torch.float64).reshape((M,) * 3)
    if verbose:
        for r, it in enumerate(its):
            print(f"Rank {r} got AC in {it} iterations.", flush=True)
        print(f"Keeping result from rank {keep}.", flush=True)
    out = ac.cpu().numpy() if numpy_io else ac
    if return_info:
        return out, {"rlambdas": rls, "flambdas": fls, "v1": v1, "v2": v2, "iterations": its, "keep": keep,
                     "solutions": [x.to(torch.float64).reshape((M,) * 3) for x in xs]}
    return out


def solve_many(solvers, ds, xs, maxiter=100, rtol=1e-5, atol=0.0):
    """Run several CGSolvers' solves together (cmt_cg_solve_many): xs (x0 in, solutions out)
    and ds are device vectors of each solver's precision.  Returns the iteration counts."""
    n = len(solvers)
    arr = lambda objs: (ctypes.c_void_p * n)(*[o for o in objs])
    hs = arr([s._h.value for s in solvers])
    dp = arr([d.data_ptr() for d in ds])
    xp = arr([x.data_ptr() for x in xs])
    its = (ctypes.c_int * n)()
    rho = (ctypes.c_double * n)()
    with torch.cuda.device(solvers[0].device):
        _lib.call("cmt_cg_solve_many", n, hs, dp, xp, int(maxiter), float(rtol), float(atol), its, rho)
    return [int(v) for v in its]


def solve_tikhonov(pixel_position_reciprocal, reciprocal_extent, slices_, M, orientations, weights=None, lam=1e-3,
                   maxiter=50, rtol=0.0, prec=32, eps=DEFAULT_EPS, operator="toeplitz", x0=None, use_graph=True,
                   return_info=False):
    """Weighted least squares with Tikhonov regularisation for the autocorrelation, on the GPU:

        argmin_x  1/(2 M^3) sum_j w_j (Re(A x)_j - b_j)^2 + lam/2 |x|^2

    with A the slicing operator of align.py:39-65 (type 2, isign -1, without its 1/M^3) at
    the rotated q-points inv(R(q)) . ppr * pi / extent, x real on M^3 modes, by CG on the
    normal equations (A^H W A / M^3 + lam I) x = Re(A^H W b) / M^3 -- the operator family of
    autocorrelation.py:113-173 (setup_linops) with weights on both sides, lam as the ridge
    term, no Fourier-domain term, and consistent scaling.  For the centrosymmetric real x an
    autocorrelation is, Re(A^H W A) x equals Re(A)^T W Re(A) x, so the CG iterates (started
    from a symmetric x0) solve the real least-squares problem.

    weights: per pixel (n_pix,) or per point (n_img * n_pix,); None means 1.
    operator "toeplitz": A^H W A as the (2M)^3 convolution with the type-1 transform of the
    weights (one spread of N weights, then no N-sized work per iteration); "pair": A^H A
    applied by the fused type-2 -> type-1 pair each iteration, recomputing the slices on the
    fly instead of storing them (unweighted only).  FP64 dot products, norms and step
    scalars in both precisions; the iteration is captured in a CUDA graph."""
    dev = torch.device("cuda", torch.cuda.current_device())
    numpy_io = not torch.is_tensor(slices_)
    Mtot = M ** 3
    rt = torch.float64 if prec == 64 else torch.float32
    ppr = _as_device(pixel_position_reciprocal, torch.float64).reshape(3, -1)
    n_pix = ppr.shape[-1]
    quats = orientations if torch.is_tensor(orientations) else np.asarray(orientations, dtype=np.float32)
    inv_rot = inverse_rotations(quats, device=dev)
    data = _as_device(slices_, torch.float32).reshape(-1)
    N = data.numel()
    w = None
    if weights is not None:
        w = _as_device(weights, torch.float64).reshape(-1)
        if w.numel() == n_pix:
            w = w.repeat(N // n_pix)
        if w.numel() != N:
            raise ValueError(f"weights must have n_pix ({n_pix}) or N ({N}) entries")
    op = PAIR if operator == "pair" else TOEPLITZ
    if op == PAIR and w is not None:
        raise ValueError("the pair operator applies unweighted A^H A; use operator='toeplitz' with weights")
    x0 = torch.zeros(Mtot, dtype=torch.float64, device=dev) if x0 is None else \
        _as_device(x0, torch.float64).reshape(-1).clone()
    ws = _workspace(M, prec, op, eps, dev)
    solver, plan_M, plan_2M = ws.solver, ws.plan_M, ws.plan_2M
    ones = torch.ones(Mtot, dtype=torch.float32, device=dev)
    # W = alambda * A^H W A / (8 M^3) (the Toeplitz kernel and the pair carry 1/(2M)^3) + lam I
    solver.set_operator(ones, 8.0, float(lam), 0.0)
    plan_M.set_pts_quat(inv_rot, ppr, float(reciprocal_extent))
    if op == TOEPLITZ:
        M2 = 2 * M
        kern = plan_2M.execute(None if w is None else w.to(rt), scale=1.0 / float(M2) ** 3, real_out=True,
                               fft_order=True)
        solver.set_kernel(kern)
    else:
        solver.set_pair_plan(plan_M)
    wb = data.to(torch.float64) * w if w is not None else data
    adb = plan_M.execute(wb.to(rt), scale=1.0 / float(M) ** 3, real_out=True).reshape(-1)
    d = adb.to(torch.float64)
    x, iters = solver.solve(d, x0, maxiter=maxiter, rtol=rtol, use_graph=use_graph)
    out = x.to(torch.float64).reshape((M,) * 3)
    out = out.cpu().numpy() if numpy_io else out
    if return_info:
        return out, {"iterations": iters, "d": d}
    return out
