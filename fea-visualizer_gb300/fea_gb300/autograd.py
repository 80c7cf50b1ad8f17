"""torch.autograd bridge of the hand-written adjoints.

`advdiff_loss(solver, u0, D, target, nsteps, checkpoint_every)` returns
J = 1/2 |u_N - target|_M^2 of the explicit advection-diffusion model on one
handle (fea_adjoint_advdiff_device) as a differentiable scalar in u0
(unknown-indexed [N]) and the per-element diffusivity D ([T]).

`gray_scott_loss(solver, u0, v0, theta, target_u, target_v, nsteps,
checkpoint_every)` returns the Gray-Scott loss (fea_adjoint_gray_scott_device)
as a differentiable scalar in u0, v0 and theta = (F, k, Du, Dv).

The forward pass runs the library's adjoint as well and keeps its gradients
for the backward pass; nothing is recorded on torch's tape, so the gradients
are the adjoint's, not autograd's.
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


class GrayScottLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u0, v0, theta, solver, target_u, target_v, nsteps, checkpoint_every):
        p = solver.params
        p.rd_feed_rate, p.rd_kill_rate, p.rd_Du, p.rd_Dv = (float(x) for x in theta.detach().cpu())
        solver.set_params(p)
        J, gu, gv, gp = solver.adjoint_gray_scott_device(u0, v0, target_u, target_v, nsteps, checkpoint_every)
        ctx.save_for_backward(gu.to(u0.dtype), gv.to(v0.dtype), torch.tensor(gp, dtype=theta.dtype,
                                                                             device=theta.device))
        return torch.tensor(J, dtype=torch.float64, device=u0.device)

    @staticmethod
    def backward(ctx, gJ):
        gu, gv, gp = ctx.saved_tensors
        return (gJ.to(gu.dtype) * gu, gJ.to(gv.dtype) * gv, gJ.to(gp.dtype).to(gp.device) * gp,
                None, None, None, None, None)


def gray_scott_loss(solver, u0, v0, theta, target_u, target_v, nsteps: int, checkpoint_every: int):
    """theta = (F, k, Du, Dv); the handle holds them as floats (the reference's parameter type)."""
    return GrayScottLoss.apply(u0, v0, theta, solver, target_u, target_v, int(nsteps), int(checkpoint_every))
