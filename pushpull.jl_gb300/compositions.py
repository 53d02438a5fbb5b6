"""Compositions of deformations on the native pull (src/compositions.jl:1-52).

``compose(ϕ, θ)`` samples the three components of ϕ at θ: one multi-channel
pull, degree 1, extrapolated, component k with a DST-II (antisymmetric)
boundary along axis k and DCT-II along the other two (the reference's boundary
matrix [2 1 1; 1 2 1; 1 1 2]).  ``Exp(v)`` follows the reference's recursion
exactly: u = v / 2^8, then eight times u = compose(u, id + u) (u resampled at
id + u; the reference adds no u term, so |u| stays near |v| / 2^8), then
id + u.  ``ExpPlan`` captures those eight steps once as a CUDA graph and
replays them (the chain is launch-bound on small grids).
"""
from __future__ import annotations

import torch

from . import layout as L
from .api import id as identity
from .api import pull
from .settings import Settings

COMPOSE_SETTINGS = Settings(1, ((2, 1, 1), (1, 2, 1), (1, 1, 2)), True)
EXP_STEPS = 8


def compose(phi: torch.Tensor, theta: torch.Tensor, *, out=None) -> torch.Tensor:
    """ψ = ϕ ∘ θ for (d…, 3) deformations (src/compositions.jl:8-39)."""
    assert phi.dim() == 4 and phi.shape[3] == 3, "`ϕ` must have three channels"
    assert theta.dim() == 4 and theta.shape[3] == 3, "`θ` must have three channels"
    return pull(phi, theta, COMPOSE_SETTINGS, out=out)


def Exp(v: torch.Tensor) -> torch.Tensor:  # noqa: N802 (the reference's name)
    """Exponentiate a stationary velocity field ``v (d…, 3)`` (src/compositions.jl:42-50)."""
    Id = identity(v)
    u = v / float(2 ** EXP_STEPS)
    for _ in range(EXP_STEPS):
        u = compose(u, Id + u)
    return u + Id


class ExpPlan:
    """``Exp`` for a fixed grid, captured once as a CUDA graph: ``plan(v)`` copies
    v into the plan's input buffer, replays the graph and returns the result
    buffer (overwritten by the next call)."""

    def __init__(self, dim, device="cuda"):
        dim = tuple(int(d) for d in dim)
        self.v = L.zeros(dim + (3,), device=device)
        self.Id = identity(dim=dim, device=device)
        self.u = L.empty(dim + (3,), device=device)
        self.w = L.empty(dim + (3,), device=device)
        self.t = L.empty(dim + (3,), device=device)
        self.out = L.empty(dim + (3,), device=device)
        side = torch.cuda.Stream(device=device)
        side.wait_stream(torch.cuda.current_stream(device))
        with torch.cuda.stream(side):
            self._chain()                       # warm-up outside the capture
        torch.cuda.current_stream(device).wait_stream(side)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self._chain()

    def _chain(self):
        torch.mul(self.v, 1.0 / float(2 ** EXP_STEPS), out=self.u)
        for _ in range(EXP_STEPS):
            torch.add(self.Id, self.u, out=self.w)
            compose(self.u, self.w, out=self.t)
            self.u.copy_(self.t)
        torch.add(self.u, self.Id, out=self.out)

    def __call__(self, v: torch.Tensor) -> torch.Tensor:
        self.v.copy_(v)
        self.graph.replay()
        return self.out
