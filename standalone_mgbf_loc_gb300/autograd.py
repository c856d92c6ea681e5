"""torch.autograd.Function over libmgbf's hand-written adjoint chain.

y = L(a) x with L = Bz sum_g P_g B_g a_g B_g R_g Bz^T (filtering_procedure).
Backward returns dL/dx = L^T gy and dL/da_g = sum u_g * v_g with
u_g = B_g R_g Bz^T x and v_g = B_g R_g Bz^T gy, computed by
mgbf_apply_with_weight_grads; the coarse generations of x are recomputed in
the backward instead of being stored by the forward.
"""
from __future__ import annotations

import torch

from .mgbf import MGBF


class MGBFFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x: torch.Tensor, weights: torch.Tensor, op: MGBF, mg_filt: int):
        op.set_weights(weights.detach().double().cpu().tolist())
        y = x.detach().contiguous().clone()
        op.filtering_procedure(mg_filt, y)
        ctx.save_for_backward(x, weights)
        ctx.op = op
        ctx.mg_filt = mg_filt
        return y

    @staticmethod
    def backward(ctx, gy: torch.Tensor):
        x, weights = ctx.saved_tensors
        op = ctx.op
        op.set_weights(weights.detach().double().cpu().tolist())
        gx, ga = op.apply_with_weight_grads(ctx.mg_filt, x.detach().contiguous(), gy.detach().contiguous())
        gw = torch.as_tensor(ga, dtype=weights.dtype, device=weights.device)
        return gx, gw, None, None


def mgbf_apply(op: MGBF, x: torch.Tensor, weights: torch.Tensor, mg_filt: int = 1) -> torch.Tensor:
    """Differentiable filtering_procedure(mg_filt) with per-generation weights."""
    return MGBFFunction.apply(x, weights, op, mg_filt)
