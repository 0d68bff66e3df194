"""Differentiable impedance misfit for inversion loops (torch.autograd).

``sigma_misfit(sigma, plan, zobs)`` and ``log_sigma_misfit(log_sigma, plan,
zobs)`` return the least-squares impedance misfit of one model as a torch
scalar.  The forward pass is one batched forward solve of the plan (all
frequencies x polarisations); its fields stay in the plan's device memory as
the checkpoint that the backward pass reads.  The backward pass is one
adjoint solve per frequency and polarisation (same operator, smoother,
corrections and precision, ``sfdx_plan_misfit_grad``) and the fused per-cell
contraction of forward and adjoint fields.  Everything runs in the native
library; tensors on a CUDA device are handed over by pointer on torch's
current stream, host tensors are copied.

The reference has no inversion path: this is the differentiation part of the
forward-solve interface.  The Dirichlet data (the 1-D background of cell
column (1,1)) are held fixed, so the gradient of the cells of that column
omits their effect through the boundary values.
"""
from __future__ import annotations

import numpy as np
import torch

from .solver import Plan


def _check(t: torch.Tensor, shape, what: str) -> None:
    """The conductivity tensor must have exactly the plan's layout: the library copies
    6 x ncell values from its storage."""
    if tuple(t.shape) != tuple(shape):
        raise ValueError(f"{what} has shape {tuple(t.shape)}, expected {tuple(shape)}")
    if t.is_cuda and torch.cuda.current_device() != t.device.index:
        raise ValueError(f"{what} is on {t.device}, the plan on cuda:{torch.cuda.current_device()}")


def _bind_stream(plan: Plan, t: torch.Tensor) -> None:
    plan.set_stream(torch.cuda.current_stream(t.device).cuda_stream if t.is_cuda else None)


def _forward(plan: Plan, sigma6: torch.Tensor, zobs, wts) -> float:
    _bind_stream(plan, sigma6)
    if sigma6.is_cuda:
        s = sigma6.detach().to(torch.float64).contiguous()
        plan.solve(sigma_device_ptr=s.data_ptr(), fetch=False)
    else:
        plan.solve(sigma=sigma6.detach().to(torch.float64).numpy(), fetch=False)
    mis, _, _, _, _ = plan.misfit_grad(zobs, wts, with_grad=False)
    return mis


def _gradient(plan: Plan, like: torch.Tensor, zobs, wts) -> torch.Tensor:
    _bind_stream(plan, like)
    m = plan.model
    if like.is_cuda:
        g = torch.empty((6, m.ncell), dtype=torch.float64, device=like.device)
        plan.misfit_grad(zobs, wts, grad_device_ptr=g.data_ptr())
        return g
    _, g, _, _, _ = plan.misfit_grad(zobs, wts)
    return torch.from_numpy(g)


class SigmaMisfit(torch.autograd.Function):
    """misfit(sigma[6, ncell]) (xx, yy, zz, xy, xz, yz per cell)."""

    @staticmethod
    def forward(ctx, sigma, plan, zobs, wts):
        _check(sigma, (6, plan.model.ncell), "sigma")
        ctx.plan, ctx.zobs, ctx.wts = plan, zobs, wts
        ctx.save_for_backward(sigma)
        mis = _forward(plan, sigma, zobs, wts)
        return torch.tensor(mis, dtype=torch.float64, device=sigma.device)

    @staticmethod
    def backward(ctx, gout):
        (sigma,) = ctx.saved_tensors
        g = _gradient(ctx.plan, sigma, ctx.zobs, ctx.wts).to(sigma.dtype)
        return gout * g, None, None, None


class LogSigmaMisfit(torch.autograd.Function):
    """misfit(log sigma[ncell]) of an isotropic model (sigma_xx = sigma_yy = sigma_zz = exp(log sigma))."""

    @staticmethod
    def forward(ctx, log_sigma, plan, zobs, wts):
        _check(log_sigma, (plan.model.ncell,), "log_sigma")
        sig = torch.exp(log_sigma.detach().to(torch.float64))
        s6 = torch.zeros((6, sig.numel()), dtype=torch.float64, device=sig.device)
        s6[0:3] = sig
        ctx.plan, ctx.zobs, ctx.wts = plan, zobs, wts
        ctx.save_for_backward(sig)
        mis = _forward(plan, s6, zobs, wts)
        return torch.tensor(mis, dtype=torch.float64, device=log_sigma.device)

    @staticmethod
    def backward(ctx, gout):
        (sig,) = ctx.saved_tensors
        g = _gradient(ctx.plan, sig, ctx.zobs, ctx.wts)
        return gout * sig * (g[0] + g[1] + g[2]), None, None, None


def sigma_misfit(sigma: torch.Tensor, plan: Plan, zobs, wts=None) -> torch.Tensor:
    return SigmaMisfit.apply(sigma, plan, np.asarray(zobs, np.float64), wts)


def log_sigma_misfit(log_sigma: torch.Tensor, plan: Plan, zobs, wts=None) -> torch.Tensor:
    return LogSigmaMisfit.apply(log_sigma, plan, np.asarray(zobs, np.float64), wts)
