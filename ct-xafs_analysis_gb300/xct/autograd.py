"""The forward projector and its exact adjoint as a differentiable pair for PyTorch.

``project(x, plan)`` is A x (libxct ``xct_fwd``: the reference forward model of
``reconstShare.cl:213-241``, bilinear ray sums over all angles), with the backward pass
A^T g computed by ``xct_adj``; ``backproject(y, plan)`` is A^T y with backward A g.  Both run
on the CUDA stream torch is using.  x is [dN][ny][nx], y is [dN][pa][px], float32, on the GPU.

``unrolled_gradient_descent`` unrolls x_{k+1} = max(x_k - step * A^T(A x_k - y), 0) and can
checkpoint every iteration (recomputing it in the backward pass), so the memory of a long
unrolled reconstruction is one iterate per step instead of all intermediate projections.
"""
import torch
from torch.utils.checkpoint import checkpoint


class _Project(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, plan):
        x = x.contiguous()
        out = torch.empty((x.shape[0], plan.pa, plan.px), device=x.device, dtype=torch.float32)
        plan.fwd(x, out)
        ctx.plan = plan
        return out

    @staticmethod
    def backward(ctx, g):
        plan = ctx.plan
        g = g.contiguous()
        gx = torch.empty((g.shape[0], plan.ny, plan.nx), device=g.device, dtype=torch.float32)
        plan.adj(g, gx)
        return gx, None


class _Backproject(torch.autograd.Function):
    @staticmethod
    def forward(ctx, y, plan):
        y = y.contiguous()
        out = torch.empty((y.shape[0], plan.ny, plan.nx), device=y.device, dtype=torch.float32)
        plan.adj(y, out)
        ctx.plan = plan
        return out

    @staticmethod
    def backward(ctx, g):
        plan = ctx.plan
        g = g.contiguous()
        gy = torch.empty((g.shape[0], plan.pa, plan.px), device=g.device, dtype=torch.float32)
        plan.fwd(g, gy)
        return gy, None


def project(x, plan):
    """A x, differentiable (backward: A^T)."""
    return _Project.apply(x, plan)


def backproject(y, plan):
    """A^T y, differentiable (backward: A)."""
    return _Backproject.apply(y, plan)


def poisson_nll(x, y, plan, eps=1e-12):
    """Poisson negative log-likelihood sum(Ax - y log Ax) of image x for counts-like data y."""
    p = project(x, plan)
    return (p - y * torch.log(p.clamp_min(eps))).sum()


def unrolled_gradient_descent(x0, y, plan, step, iters, checkpoint_each=True):
    """iters steps of projected gradient descent on 0.5 ||A x - y||^2; differentiable in
    x0, y and step.  With checkpoint_each, every iteration is recomputed in the backward
    pass instead of being stored."""

    def one(x, yy, st):
        r = project(x, plan) - yy
        return torch.clamp(x - st * backproject(r, plan), min=0.0)

    x = x0
    for _ in range(iters):
        if checkpoint_each:
            x = checkpoint(one, x, y, step, use_reentrant=False)
        else:
            x = one(x, y, step)
    return x
