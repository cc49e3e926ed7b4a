"""torch.autograd bridge for the misfit gradient: a thin harness over the
C-ABI's awe_gradient, so the gradient can be checked (and used) from torch.

    J = misfit(m, plan, wav, dobs)     # m = 1/v^2, model shape, any device
    J.backward()                       # m.grad = dJ/dm from the adjoint

The plan's model is replaced by 1/sqrt(m) on every call (its one-way ABC
coefficients follow the model; the gradient holds them fixed).
"""
from __future__ import annotations

import torch

from .engine import CKPT_BFP16


class MisfitFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, m, plan, wav, dobs, ckpt_every, ckpt_format):
        v = (1.0 / torch.sqrt(m.detach().to(torch.float64))).to(torch.float32).cpu().numpy()
        plan.set_model(v)
        grad, J = plan.gradient(wav, dobs, ckpt_every=ckpt_every, ckpt_format=ckpt_format)
        ctx.save_for_backward(torch.from_numpy(grad).to(device=m.device, dtype=m.dtype))
        return torch.tensor(J, dtype=m.dtype, device=m.device)

    @staticmethod
    def backward(ctx, gJ):
        (g,) = ctx.saved_tensors
        return gJ * g, None, None, None, None, None


def misfit(m, plan, wav, dobs, ckpt_every: int = 0, ckpt_format: int = CKPT_BFP16):
    """0.5 ||d(m) - dobs||^2 as a differentiable scalar of m = 1/v^2."""
    return MisfitFunction.apply(m, plan, wav, dobs, ckpt_every, ckpt_format)
