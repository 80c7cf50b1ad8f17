"""torch.autograd bridge of the hand-written adjoint (fea_adjoint_advdiff_device).

`advdiff_loss(solver, u0, D, target, nsteps, checkpoint_every)` returns
J = 1/2 |u_N - target|_M^2 of the explicit advection-diffusion model on one
handle as a differentiable scalar in u0 (unknown-indexed [N]) and the
per-element diffusivity D ([T]).  The forward pass runs the library's adjoint
as well and keeps its gradients for the backward pass; nothing is recorded
on torch's tape, so the gradients are the adjoint's, not autograd's.
"""
from __future__ import annotations

import torch


class AdvDiffLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u0, D, solver, target, nsteps, checkpoint_every):
        solver.set_element_diffusivity_device(D)
        J, gu, gD = solver.adjoint_advdiff_device(u0, target, nsteps, checkpoint_every)
        ctx.save_for_backward(gu.to(u0.dtype), gD.to(D.dtype))
        return torch.tensor(J, dtype=torch.float64, device=u0.device)

    @staticmethod
    def backward(ctx, gJ):
        gu, gD = ctx.saved_tensors
        return gJ.to(gu.dtype) * gu, gJ.to(gD.dtype) * gD, None, None, None, None


def advdiff_loss(solver, u0, D, target, nsteps: int, checkpoint_every: int):
    return AdvDiffLoss.apply(u0, D, solver, target, int(nsteps), int(checkpoint_every))
