"""Differentiable NUFFT for torch: gradients w.r.t. the image/k-space data and
w.r.t. the trajectory.

``nufft_forward(x, om, op)`` and ``nufft_adjoint(y, om, op)`` are autograd
functions over a planned ``NUFFT`` ``op``.  Their backward passes are the
hand-written adjoint/forward transforms:

* y = A x (forward, unnormalised):      dL/dx = A^H g = prod(Kd) * op.adjoint(g)
* x = op.adjoint(y) = A^H y / prod(Kd): dL/dy = op.forward(g) / prod(Kd)

(torch's complex convention: the incoming gradient g is the conjugate
Wirtinger derivative, so a linear map's backward is its Hermitian adjoint).

Trajectory gradients use the derivative of the exact NUDFT,
dy_m/d om_{m,d} = sum_n x_n (-i (n_d - N_d/2)) exp(-i om_m . (n - N/2)),
evaluated by the NUFFT of (-i (n_d - N_d/2)) x (``op.forward_dom``); the
interpolator's own dependence on om (through floor and the min-max fit) is
not differentiated.  For a real loss, dL/d om_{m,d} = Re(conj(g_m) dy_m/d om_{m,d})
summed over coils.  The adjoint's trajectory gradient follows from the same
derivative with the roles of image and samples exchanged.

When ``om`` changes between calls (trajectory optimisation) the op is
re-planned on the device from the new points before the transform.
"""
from __future__ import annotations

import torch
from torch.utils.checkpoint import checkpoint


def _sync_points(op, om):
    """Re-plan `op` if `om` is not the point set it was planned with."""
    key = (om.data_ptr(), om._version, tuple(om.shape))
    if getattr(op, '_om_key', None) != key:
        op.plan(om.detach(), op.Nd, op.Kd, op.Jd, batch=op.batch,
                deterministic=getattr(op, 'deterministic', False))
        op._om_key = key


class _Forward(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, om, op):
        if om is not None:
            _sync_points(op, om)
        ctx.op = op
        ctx.save_for_backward(x)
        ctx.has_om = om is not None
        ctx.om_dtype = om.dtype if om is not None else None
        return op.forward(x.contiguous())

    @staticmethod
    def backward(ctx, g):
        op = ctx.op
        (x,) = ctx.saved_tensors
        g = g.contiguous().to(torch.complex64)
        gx = gom = None
        if ctx.needs_input_grad[0]:
            gx = op.adjoint(g) * float(op.Kdprod)
        if ctx.has_om and ctx.needs_input_grad[1]:
            dy = op.forward_dom(x.detach().contiguous())         # (d, M[, B])
            t = torch.real(torch.conj(g).unsqueeze(0) * dy)
            if t.dim() == 3:
                t = t.sum(-1)
            gom = t.transpose(0, 1).to(ctx.om_dtype)
        return gx, gom, None


class _Adjoint(torch.autograd.Function):
    @staticmethod
    def forward(ctx, y, om, op):
        if om is not None:
            _sync_points(op, om)
        ctx.op = op
        ctx.save_for_backward(y)
        ctx.has_om = om is not None
        ctx.om_dtype = om.dtype if om is not None else None
        return op.adjoint(y.contiguous())

    @staticmethod
    def backward(ctx, g):
        op = ctx.op
        (y,) = ctx.saved_tensors
        g = g.contiguous().to(torch.complex64)
        gy = gom = None
        if ctx.needs_input_grad[0]:
            gy = op.forward(g) / float(op.Kdprod)
        if ctx.has_om and ctx.needs_input_grad[1]:
            # x_n = (1/K) sum_m y_m exp(+i om_m.(n-N/2)):
            # dL/d om_{m,d} = Re(y_m conj(D_d[g]_m)) / K with D_d the forward derivative
            dg = op.forward_dom(g)                                  # (d, M[, B])
            t = torch.real(y.detach().unsqueeze(0) * torch.conj(dg)) / float(op.Kdprod)
            if t.dim() == 3:
                t = t.sum(-1)
            gom = t.transpose(0, 1).to(ctx.om_dtype)
        return gy, gom, None


def nufft_forward(x, om, op):
    """Differentiable y = op.forward(x); pass om=None to keep the planned points
    fixed (no trajectory gradient)."""
    return _Forward.apply(x, om, op)


def nufft_adjoint(y, om, op):
    """Differentiable x = op.adjoint(y) (scaled by 1/prod(Kd) like the reference)."""
    return _Adjoint.apply(y, om, op)


def normal(x, op):
    """A^H A x with the reference's adjoint scaling (op.selfadjoint), differentiable."""
    return nufft_adjoint(nufft_forward(x, None, op), None, op)


def cg_unrolled(op, y, iters: int = 10, checkpoint_each: bool = True, lam: float = 0.0):
    """Image-domain CG on (A^H A / prod(Kd) + lam) x = A^H y / prod(Kd), x0 = 0,
    unrolled for `iters` iterations and differentiable end to end.  With
    `checkpoint_each` every iteration is an activation checkpoint: the backward
    pass recomputes one iteration at a time instead of storing all of them."""
    b = nufft_adjoint(y, None, op)
    x = torch.zeros_like(b)
    r = b.clone()
    p = r.clone()
    rs = torch.real(torch.vdot(r.flatten(), r.flatten()))

    def one(x, r, p, rs):
        Ap = normal(p, op) + lam * p
        alpha = rs / torch.real(torch.vdot(p.flatten(), Ap.flatten()))
        x = x + alpha * p
        r = r - alpha * Ap
        rs_new = torch.real(torch.vdot(r.flatten(), r.flatten()))
        p = r + (rs_new / rs) * p
        return x, r, p, rs_new

    for _ in range(iters):
        if checkpoint_each and torch.is_grad_enabled():
            x, r, p, rs = checkpoint(one, x, r, p, rs, use_reentrant=False)
        else:
            x, r, p, rs = one(x, r, p, rs)
    return x
