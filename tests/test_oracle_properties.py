"""Properties of the FP64 oracle that the reference's own tests check
(test/runtests.jl:34-96): gradients against central finite differences and the
push/pull adjoint identity, plus the same identity for pull_grad / push_grad."""
from __future__ import annotations

import itertools

import numpy as np
import pytest


def _inputs(O, rng, d=(8, 7, 1), c=2, b=None, sigma=1.0):
    shape_f = d + (c,) + ((b,) if b else ())
    f1 = np.asfortranarray(rng.standard_normal(shape_f).astype(np.float32))
    f2 = np.asfortranarray(rng.standard_normal(shape_f).astype(np.float32))
    if b:
        phi = np.stack([O.identity(d) + sigma * rng.standard_normal(d + (3,)).astype(np.float32)
                        for _ in range(b)], axis=-1)
    else:
        phi = O.identity(d) + sigma * rng.standard_normal(d + (3,)).astype(np.float32)
    return f1, f2, np.asfortranarray(phi.astype(np.float32))


@pytest.mark.parametrize("deg,bnd,ext", list(itertools.product(range(5), [0, 1, 2, (0, 1, 2)], [0, 1])))
def test_adjoint_identity(O, deg, bnd, ext):
    """|<f1, pull(f2)> - <push(f1), f2>| small; the reference uses 1e-5 absolute (test/runtests.jl:93-95)."""
    rng = np.random.default_rng(100 + deg)
    s = O.Sett.make(deg, bnd, ext)
    f1, f2, phi = _inputs(O, rng, d=(9, 7, 5), c=2, sigma=1.5)
    lhs = np.nansum(f1.astype(np.float64) * O.pull(f2, phi, s))
    rhs = np.sum(O.push(f1, phi, f2.shape[:3], s) * f2)
    assert abs(lhs - rhs) <= 1e-10 * max(1.0, abs(lhs))
    g = np.asfortranarray(rng.standard_normal((9, 7, 5, 3, 2)).astype(np.float32))
    lhs = np.nansum(g.astype(np.float64) * O.pull_grad(f2, phi, s))
    rhs = np.sum(O.push_grad(g, phi, f2.shape[:3], s) * f2)
    assert abs(lhs - rhs) <= 1e-10 * max(1.0, abs(lhs))


def _fd_phi_pull(O, f1, f2, phi, s):
    """d/dphi of sum((pull(f1,phi)-f2)^2) by central differences (eps 0.01, test/utils.jl:7)."""
    g = np.zeros(phi.shape)
    p = phi.copy(order="F")
    for idx in np.ndindex(phi.shape):
        x0 = p[idx]
        p[idx] = np.float32(x0 + np.float32(0.01))
        hp = float(p[idx]) - float(x0)
        ep = np.nansum((O.pull(f1, p, s) - f2) ** 2)
        p[idx] = np.float32(x0 - np.float32(0.01))
        hm = float(x0) - float(p[idx])
        em = np.nansum((O.pull(f1, p, s) - f2) ** 2)
        p[idx] = x0
        g[idx] = (ep - em) / (hp + hm)
    return g


@pytest.mark.parametrize("deg", [2, 3])
def test_fd_gradient_wrt_phi(O, deg):
    """Analytic d/dphi (the pull rrule: sum_c delta * pull_grad, src/pushpull_pb.jl:11-18)
    against central differences; relative squared error below 1e-3 as in test/runtests.jl:63-73."""
    rng = np.random.default_rng(7 + deg)
    s = O.Sett.make(deg, (0, 1, 2), 1)
    f1, f2, phi = _inputs(O, rng)
    r = O.pull(f1, phi, s) - f2                              # (d, C)
    gr = O.pull_grad(f1, phi, s)                              # (d, 3, C)
    ana = np.einsum("xyzc,xyzkc->xyzk", 2 * r, gr)
    fd = _fd_phi_pull(O, f1, f2, phi, s)
    assert np.sum((ana - fd) ** 2) / np.sum(ana ** 2) < 1e-3


@pytest.mark.parametrize("deg", [3, 4])
def test_hessian_is_jacobian_of_gradient(O, deg):
    """pull_hess against central differences of pull_grad in the sample position
    (the pair the pull_grad rrule chains, src/pushpull_pb.jl:26-35): splines of
    degree 3 and 4 are C^2, positions inside the image, two channels with
    different bounds; relative error below 1e-3."""
    rng = np.random.default_rng(40 + deg)
    d = (11, 10, 9)
    f = np.asfortranarray(rng.standard_normal(d + (2,)).astype(np.float32))
    phi = np.empty(d + (3,), dtype=np.float32, order="F")
    for k in range(3):
        phi[..., k] = rng.uniform(3.0, d[k] - 2.0, d).astype(np.float32)
    s = O.Sett.make(deg, [(1, 1, 1), (2, 0, 1)], 1)
    H = O.pull_hess(f, phi, s)                                # (d, 3, 3, C)
    assert np.allclose(H, np.swapaxes(H, 3, 4), rtol=0, atol=1e-10 * np.abs(H).max())
    fd = np.zeros_like(H)
    for q in range(3):
        pp, pm = phi.copy(order="F"), phi.copy(order="F")
        pp[..., q] = (phi[..., q] + np.float32(0.002)).astype(np.float32)
        pm[..., q] = (phi[..., q] - np.float32(0.002)).astype(np.float32)
        step = (pp[..., q].astype(np.float64) - pm[..., q].astype(np.float64))[..., None, None]
        fd[..., :, q, :] = ((O.pull_grad(f, pp, s) - O.pull_grad(f, pm, s)) / step)
    assert np.sqrt(np.sum((H - fd) ** 2) / np.sum(H ** 2)) < 1e-3
