"""The reference's own test set (test/runtests.jl:37-98, test/utils.jl:3-25),
restated for the torch autograd rules on the GB300 kernels.

A small (8, 7, 1) grid with two channels and a deformation of identity plus
N(0, 1) noise.  For degrees 2 and 3 with bounds (circulant, DCT-II, DST-II),
the analytic gradient of a squared-error loss through pull, push and pull_grad
is compared with central differences (step 0.01 on every element).  The
criterion is the reference's: sum((g - g_fd)^2) / sum(g^2) < 1e-3.  Batch size
two at degree 3, and the push/pull adjoint to 1e-5 (relative once the sums exceed 1).  Losses are summed
in float64; the seeds replace the reference's unseeded randn."""
from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = 1e-3
D = (8, 7, 1)


def _grad_check(fun, theta):
    """The reference's test_grad: autograd gradient against central differences."""
    t = theta.detach().clone().requires_grad_(True)
    fun(t).backward()
    g0 = t.grad.detach().double()
    num = torch.zeros_like(g0)
    base = theta.detach().clone()
    idx = np.ndindex(*base.shape)
    eps = 0.01
    with torch.no_grad():
        for i in idx:
            x0 = float(base[i])
            base[i] = x0 + eps
            ep = float(fun(base))
            base[i] = x0 - eps
            em = float(fun(base))
            base[i] = x0
            num[i] = (ep - em) / (2 * eps)
    return float(((g0 - num) ** 2).sum() / (g0 ** 2).sum())


def _data(pkg, seed, bs=None):
    L = pkg.layout
    g = torch.Generator(device="cuda").manual_seed(seed)
    tail = (2,) if bs is None else (2, bs)
    f1 = L.empty(D + tail)
    f2 = L.empty(D + tail)
    phi = L.empty(D + ((3,) if bs is None else (3, bs)))
    for t in (f1, f2, phi):
        L.flat(t).copy_(torch.randn(t.numel(), generator=g, device="cuda"))
    ident = pkg.id(dim=D)
    with torch.no_grad():
        if bs is None:
            phi += ident
        else:
            phi += ident.unsqueeze(-1)
    return f1, f2, phi


def _sse(x, y):
    return ((x.double() - y.double()) ** 2).sum()


@pytest.mark.parametrize("deg", [2, 3])
def test_pull_push_gradients(pkg, deg):
    A = pkg.autograd
    s = pkg.Settings((deg,) * 3, (0, 1, 2), True)
    f1, f2, phi = _data(pkg, 10 + deg)
    assert _grad_check(lambda th: _sse(A.pull(f1, th, s), f2), phi) < TOL
    assert _grad_check(lambda th: _sse(A.pull(th, phi, s), f2), f1) < TOL
    assert _grad_check(lambda th: _sse(A.push(f1, th, D, s), f2), phi) < TOL
    assert _grad_check(lambda th: _sse(A.push(th, phi, D, s), f2), f1) < TOL
    if deg == 3:
        g2 = pkg.pull_grad(f2, phi, s)
        assert _grad_check(lambda th: _sse(A.pull_grad(f1, th, s), g2), phi) < TOL


def test_batch_of_two_and_adjoint(pkg):
    A = pkg.autograd
    s = pkg.Settings((3, 3, 3), (0, 1, 2), True)
    f1, f2, phi = _data(pkg, 20, bs=2)
    assert _grad_check(lambda th: _sse(A.pull(f1, th, s), f2), phi) < TOL
    assert _grad_check(lambda th: _sse(A.pull(th, phi, s), f2), f1) < TOL
    assert _grad_check(lambda th: _sse(A.push(f1, th, D, s), f2), phi) < TOL
    assert _grad_check(lambda th: _sse(A.push(th, phi, D, s), f2), f1) < TOL
    lhs = float((f1.double() * pkg.pull(f2, phi, s).double()).sum())
    rhs = float((pkg.push(f1, phi, D, s).double() * f2.double()).sum())
    assert abs(lhs - rhs) < 1e-5 * max(1.0, abs(lhs))
