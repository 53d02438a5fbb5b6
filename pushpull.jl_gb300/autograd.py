"""Differentiation rules: torch.autograd.Function versions of the reference's
ChainRulesCore rrules (src/pushpull_pb.jl:11-51).

* ``Pull``:     ∂f₀ = push(δ),        ∂ϕ = Σ_c δ_c ∇pull(f₀_c)   (pull_grad_dot kernel)
* ``PullGrad``: ∂f₀ = push_grad(δ),   ∂ϕ = Σ_c H_c δ_c           (pull_hess_dot kernel)
* ``Push``:     ∂f₁ = pull(δ),        ∂ϕ = Σ_c f₁_c ∇pull(δ_c)   (pull_grad_dot with the roles swapped)
* ``FusedLoss``: loss = Σ(pull(f₀, ϕ) - g)² with both gradients from one fused kernel,
  evaluated in the forward pass (the "differentiable step").

Backward passes recompute from the saved inputs; no forward output is stored.
The ∂ϕ contractions never materialise the (d₁…, 3, C, B) gradient temporary the
reference builds.
"""
from __future__ import annotations

import torch

from . import api
from . import layout as L
from .settings import Settings


class Pull(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f0, phi, sett: Settings):
        ctx.save_for_backward(f0, phi)
        ctx.sett = sett
        return api.pull(f0, phi, sett)

    @staticmethod
    def backward(ctx, delta):
        f0, phi = ctx.saved_tensors
        s = ctx.sett
        delta = L.colmajor(delta)
        df = api.push(delta, phi, tuple(f0.shape[:3]), s) if ctx.needs_input_grad[0] else None
        dphi = api.pull_grad_dot(f0, phi, delta, s) if ctx.needs_input_grad[1] else None
        return df, dphi, None


class PullGrad(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f0, phi, sett: Settings):
        ctx.save_for_backward(f0, phi)
        ctx.sett = sett
        return api.pull_grad(f0, phi, sett)

    @staticmethod
    def backward(ctx, delta):
        f0, phi = ctx.saved_tensors
        s = ctx.sett
        delta = L.colmajor(delta)
        df = api.push_grad(delta, phi, tuple(f0.shape[:3]), s) if ctx.needs_input_grad[0] else None
        dphi = api.pull_hess_dot(f0, phi, delta, s) if ctx.needs_input_grad[1] else None
        return df, dphi, None


class Push(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f1, phi, d0, sett: Settings):
        ctx.save_for_backward(f1, phi)
        ctx.sett = sett
        return api.push(f1, phi, d0, sett)

    @staticmethod
    def backward(ctx, delta):
        f1, phi = ctx.saved_tensors
        s = ctx.sett
        delta = L.colmajor(delta)
        df1 = api.pull(delta, phi, s) if ctx.needs_input_grad[0] else None
        dphi = api.pull_grad_dot(delta, phi, f1, s) if ctx.needs_input_grad[1] else None
        return df1, dphi, None, None


class FusedLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f0, phi, g, sett: Settings):
        loss, df, dphi = api.fused_step(f0, phi, g, sett)
        ctx.save_for_backward(df, dphi)
        return loss

    @staticmethod
    def backward(ctx, gout):
        df, dphi = ctx.saved_tensors
        s = gout.to(torch.float32)
        return df * s, dphi * s, None, None


def pull(f0, phi, sett: Settings = Settings()):
    return Pull.apply(f0, phi, sett)


def pull_grad(f0, phi, sett: Settings = Settings()):
    return PullGrad.apply(f0, phi, sett)


def push(f1, phi, d0, sett: Settings = Settings()):
    return Push.apply(f1, phi, tuple(int(v) for v in d0), sett)


def fused_loss(f0, phi, g, sett: Settings = Settings()):
    return FusedLoss.apply(f0, phi, g, sett)
