"""Differentiable slicing: the model slices of cmtip's alignment (cmtip/alignment/align.py:39-65,
``Re(type-2 NUFFT of the autocorrelation)`` at rotated q-points) as torch autograd ops.

``Slice.apply(ac, plan2, plan1)`` returns ``c = Re(A ac)`` with ``(A f)_j = sum_k f_k e^{-i k.x_j}``
(type 2, isign -1).  Its backward is the hand-written adjoint: for a real cotangent ``g``,
``d(g.c)/d ac = Re(A^H g) = Re(sum_j g_j e^{+i k.x_j})``, a type-1 spread (isign +1) of ``g``
with real output -- the same operation as cmtip's adjoint (cmtip/nufft/adjoint.py:13-43)
without its 1/M^3.

``sliced_least_squares(ac, quats, ppr, extent, data, chunk)`` is the data term
``1/2 sum_j (Re(A ac)_j - b_j)^2`` over an image set processed ``chunk`` images at a time:
the forward keeps no slices, and the backward recomputes each chunk's slices to form its
residual, so device memory is bounded by one chunk (image sets larger than HBM).
"""
from __future__ import annotations

import torch

from .nufft import DEFAULT_EPS, Plan, inverse_rotations


class Slice(torch.autograd.Function):
    """c = Re(A f) on the points of ``plan2`` (type 2, isign -1); backward via ``plan1``
    (type 1, isign +1, same points).  ``plan1`` must keep the forward's points until the
    backward has run: giving it new points in between raises in the backward instead of
    returning the gradient on the wrong points."""

    @staticmethod
    def forward(ctx, f: torch.Tensor, plan2: Plan, plan1: Plan):
        ctx.plan1 = plan1
        ctx.points_version = plan1.points_version
        ctx.fshape = f.shape
        return plan2.execute(f.detach().reshape(-1), real_out=True)

    @staticmethod
    def backward(ctx, g: torch.Tensor):
        if ctx.plan1.points_version != ctx.points_version:
            raise RuntimeError("Slice.backward: the adjoint plan was given new points after the forward; "
                               "run backward before re-pointing the plans (or use one SlicePlans per graph)")
        grad = ctx.plan1.execute(g.detach().contiguous().reshape(-1), real_out=True)
        return grad.reshape(ctx.fshape).to(g.dtype), None, None


class SlicePlans:
    """A matched pair of plans (type 2 forward, type 1 adjoint) on the same points."""

    def __init__(self, M, prec=64, eps=DEFAULT_EPS):
        self.fwd = Plan(2, M, eps=eps, isign=-1, prec=prec)
        self.adj = Plan(1, M, eps=eps, isign=1, prec=prec)

    def set_pts(self, x, y, z):
        self.fwd.set_pts(x, y, z)
        self.adj.set_pts(x, y, z)
        return self

    def set_pts_quat(self, inv_rot, ppr, extent):
        self.fwd.set_pts_quat(inv_rot, ppr, extent)
        self.adj.set_pts_quat(inv_rot, ppr, extent)
        return self

    def __call__(self, f):
        return Slice.apply(f, self.fwd, self.adj)


class _SlicedLSQ(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f, plans, inv_rot, ppr, extent, data, chunk):
        ctx.save_for_backward(f.detach())
        ctx.args = (plans, inv_rot, ppr, extent, data, chunk)
        loss = torch.zeros((), dtype=torch.float64, device=f.device)
        n_img = inv_rot.shape[0]
        for s in range(0, n_img, chunk):
            plans.fwd.set_pts_quat(inv_rot[s:s + chunk], ppr, extent)
            c = plans.fwd.execute(f.detach().reshape(-1), real_out=True)
            r = c.double() - data[s:s + chunk].reshape(-1).to(f.device, torch.float64)
            loss += 0.5 * torch.dot(r, r)
        return loss

    @staticmethod
    def backward(ctx, gl):
        (f,) = ctx.saved_tensors
        plans, inv_rot, ppr, extent, data, chunk = ctx.args
        grad = torch.zeros(f.numel(), dtype=f.dtype, device=f.device)
        n_img = inv_rot.shape[0]
        for s in range(0, n_img, chunk):
            # recompute this chunk's slices instead of having stored them
            plans.fwd.set_pts_quat(inv_rot[s:s + chunk], ppr, extent)
            c = plans.fwd.execute(f.reshape(-1), real_out=True)
            r = (c - data[s:s + chunk].reshape(-1).to(f.device, f.dtype)).contiguous()
            plans.adj.set_pts_quat(inv_rot[s:s + chunk], ppr, extent)
            grad += plans.adj.execute(r, real_out=True).reshape(-1)
        return (grad * gl).reshape(f.shape), None, None, None, None, None, None


def sliced_least_squares(ac: torch.Tensor, quats, ppr, reciprocal_extent, data, chunk=256, prec=None,
                         eps=DEFAULT_EPS):
    """1/2 ||Re(A ac) - data||^2 over all images, ``chunk`` images resident at a time.
    ``quats`` (n, 4) float32, ``ppr`` (3, n_pix) float64, ``data`` (n, n_pix) (may stay on the
    host: each chunk is copied when it is needed)."""
    prec = prec or (64 if ac.dtype == torch.float64 else 32)
    plans = SlicePlans(ac.shape[0], prec=prec, eps=eps)
    inv = inverse_rotations(quats, device=ac.device)
    pprd = torch.as_tensor(ppr, device=ac.device, dtype=torch.float64).reshape(3, -1).contiguous()
    return _SlicedLSQ.apply(ac, plans, inv, pprd, float(reciprocal_extent), data, int(chunk))
