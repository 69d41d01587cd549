"""torch.autograd.Function for the projector log-weight.

``LogWeight.apply(x, chains)`` maps phonon fields ``x`` of shape
``[B, n_bf, Lt]`` (float64, CUDA) to ``W[b] = Re log det(P^H B(Lt..1) P)``
(cal_new_weight_T0, src/mod_evolution.f90:359-408) for every chain, and its
backward returns ``dW/dx`` from the hand-written adjoint
(``pqmc_logweight_grad``: checkpointed left factors every ngroup slices and
the Green's-function trace formula, csrc/adjoint.cu).  Each chain is a
``PqmcChain`` of matching model; its fast-update state is not disturbed.

The chains are independent: each runs on its own CUDA stream, driven from
its own host thread (the C-ABI allows one thread per chain handle), so the
small per-chain kernels of different chains overlap on the GPU.  The
thread count is ``PQMC_GRAD_THREADS`` (default: up to 8).
"""
from __future__ import annotations

import concurrent.futures as cf
import os

import torch

from .engine import PqmcChain


def _threads(n: int) -> int:
    try:
        t = int(os.environ.get("PQMC_GRAD_THREADS", "8"))
    except ValueError:
        t = 8
    return max(1, min(n, t))


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

        def one(b: int) -> float:
            ch = chains[b]
            ch.set_field_device(xf[b].data_ptr())
            ch.init_expkv()
            return ch.logweight_grad_device(grads[b].data_ptr()).real

        nt = _threads(B)
        if nt == 1:
            for b in range(B):
                vals[b] = one(b)
        else:
            with cf.ThreadPoolExecutor(max_workers=nt) as ex:
                for b, w in enumerate(ex.map(one, range(B))):
                    vals[b] = w
        ctx.save_for_backward(grads.transpose(1, 2))
        return vals.to(x.device)

    @staticmethod
    def backward(ctx, gout: torch.Tensor):
        (grads,) = ctx.saved_tensors
        return gout.to(grads.dtype)[:, None, None] * grads, None


def log_weight(x: torch.Tensor, chains: list[PqmcChain]) -> torch.Tensor:
    return LogWeight.apply(x, chains)
