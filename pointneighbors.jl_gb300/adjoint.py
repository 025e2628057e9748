"""The differentiable form: L(x) = sum_i (rho_i - 1)^2 + lambda E as a torch.autograd.Function
over the C ABI's AdjointLossForward / AdjointLossBackward pair functions.

The reference has no adjoint; in Julia this is what a `ChainRulesCore.rrule` for the
loss would bind.  The neighbour set is piecewise constant in x, so it is held fixed at the
forward's positions: the gradient is that of the loss over those pairs.  forward()
re-bins the search at x (update!) and runs the forward sweep; backward() re-traverses the
cell list (no pair list is stored) and scales by the upstream gradient on the device.  If
the search was re-binned in between (another forward, an update!), backward() first re-bins
it at the forward's positions, which it keeps a copy of.
"""
from __future__ import annotations

import torch

from . import AdjointLossBackward, AdjointLossForward, _tdtype, foreach_point_neighbor, update


class _AdjointLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, nhs, mass, h, cutoff, lambda_pot):
        n = x.shape[1]
        update(nhs, x, x, check=False)
        vt = _tdtype(nhs)  # the pair arithmetic's type (Float32 in a mixed search)
        density = torch.empty(n, dtype=vt, device=x.device)
        terms = torch.empty(n, dtype=vt, device=x.device)
        loss = torch.empty(1, dtype=torch.float64, device=x.device)
        f = AdjointLossForward(density=density, terms=terms, loss=loss, mass=mass, h=h,
                               cutoff=cutoff, lambda_pot=lambda_pot)
        foreach_point_neighbor(f, nhs._y_keep, nhs._y_keep, nhs, check=True)
        ctx.nhs = nhs
        ctx.consts = dict(mass=mass, h=h, cutoff=cutoff, lambda_pot=lambda_pot)
        ctx.generation = nhs._generation
        ctx.positions = nhs._y_keep.detach().clone()  # (d, N), strides (1, d)
        ctx.save_for_backward(density)
        return loss[0]

    @staticmethod
    def backward(ctx, g_out):
        nhs = ctx.nhs
        if nhs._generation != ctx.generation:  # re-bin at the forward's positions
            update(nhs, ctx.positions, ctx.positions, check=False)
        (density,) = ctx.saved_tensors
        y = nhs._y_keep
        n, d = y.shape[1], y.shape[0]
        grad = torch.empty(n * d, dtype=_tdtype(nhs), device=y.device)
        scale = g_out.detach().to(torch.float64).reshape(1).contiguous()
        f = AdjointLossBackward(density=density, grad=grad, grad_scale=scale,
                                reuse_state=False, **ctx.consts)
        foreach_point_neighbor(f, y, y, nhs, check=True)
        return grad.view(n, d).t().to(y.dtype), None, None, None, None, None


def adjoint_loss(x, nhs, *, mass=1.0, h=1.5, cutoff=3.0, lambda_pot=0.01):
    """L(x) = sum_i (rho_i - 1)^2 + lambda_pot * E with gradients through torch.autograd.

    `x` is a (d, N) CUDA tensor (the reference's layout); `nhs` a GridNeighborhoodSearch
    whose cell list is re-binned at x by the forward pass.  Returns a 0-d float64 tensor."""
    return _AdjointLoss.apply(x, nhs, float(mass), float(h), float(cutoff), float(lambda_pot))
