"""torch.autograd.Function for the projector log-weight.

``LogWeight.apply(x, chains)`` maps phonon fields ``x`` of shape
``[B, n_bf, Lt]`` (float64, CUDA) to ``W[b] = Re log det(P^H B(Lt..1) P)``
(cal_new_weight_T0, src/mod_evolution.f90:359-408) for every chain, and its
backward returns ``dW/dx`` from the hand-written adjoint
(``pqmc_logweight_grad``: checkpointed left factors every ngroup slices and
the Green's-function trace formula, csrc/adjoint.cu).  Each chain is a
``PqmcChain`` of matching model; its fast-update state is not disturbed.
"""
from __future__ import annotations

import torch

from .engine import PqmcChain


class LogWeight(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x: torch.Tensor, chains: list[PqmcChain]):
        if x.device.type != "cuda" or x.dtype != torch.float64:
            raise TypeError("LogWeight expects a float64 CUDA tensor [B, n_bf, Lt]")
        B = x.shape[0]
        if B != len(chains):
            raise ValueError("one chain per batch entry")
        # (n_bf, Lt) column-major == (Lt, n_bf) row-major
        xf = x.detach().transpose(1, 2).contiguous()
        grads = torch.empty_like(xf)
        vals = torch.empty(B, dtype=torch.float64)
        torch.cuda.synchronize()
        for b, ch in enumerate(chains):
            ch.set_field_device(xf[b].data_ptr())
            ch.init_expkv()
            ch.init_g(1)
            w = ch.logweight_grad_device(grads[b].data_ptr())
            vals[b] = w.real
        ctx.save_for_backward(grads.transpose(1, 2))
        return vals.to(x.device)

    @staticmethod
    def backward(ctx, gout: torch.Tensor):
        (grads,) = ctx.saved_tensors
        return gout.to(grads.dtype)[:, None, None] * grads, None


def log_weight(x: torch.Tensor, chains: list[PqmcChain]) -> torch.Tensor:
    return LogWeight.apply(x, chains)
