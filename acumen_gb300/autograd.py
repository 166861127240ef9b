"""torch.autograd binding of the registration-aware TV objective, used by the
gradient-check harness only: forward and backward both call the C ABI's
hand-written kernels (acu_tv_loss_grad_dev / _f64); torch does no arithmetic
on the path."""
from __future__ import annotations

import torch


class TVObjective(torch.autograd.Function):
    """loss = sum_s 1/2 |A_off u_s - y_s|^2 + lambda TV_eps(u_s)."""

    @staticmethod
    def forward(ctx, u, off, y, tomo, lam, eps):
        loss, gu, go = tomo.tv_loss_grad(u, off, y, lam, eps, want_grad=True)
        ctx.save_for_backward(gu, go if go is not None else torch.empty(0, device=u.device))
        ctx.has_off = go is not None
        return torch.as_tensor(float(loss.sum()), dtype=u.dtype, device=u.device)

    @staticmethod
    def backward(ctx, gout):
        gu, go = ctx.saved_tensors
        return (gout * gu, (gout * go) if ctx.has_off else None, None, None, None, None)


def tv_objective(tomo, u, off, y, lam, eps):
    return TVObjective.apply(u, off, y, tomo, lam, eps)
