"""Differentiation: the ϕ-cotangent contraction kernels, the fused forward+adjoint
step, and the autograd rules (the reference rrules, src/pushpull_pb.jl:11-51),
against the FP64 oracle and central finite differences.

Tolerances (norm-wise relative, NaN masks identical):
  contractions, fused df / dphi      1e-4 vs FP64 oracle
  fused loss                         1e-5 vs FP64 oracle
  finite differences (h = 1e-3 vox)  1e-3 (the reference's criterion, test/runtests.jl:42)
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _phi(O, rng, d1, d0, sigma, nb=None):
    def one():
        p = O.identity(d1).astype(np.float64)
        for k in range(3):
            p[..., k] = 1 + (p[..., k] - 1) * (d0[k] - 1) / max(d1[k] - 1, 1)
        return p + sigma * rng.standard_normal(p.shape)
    a = np.stack([one() for _ in range(nb)], axis=-1) if nb else one()
    return np.asfortranarray(a.astype(np.float32))


def _f(rng, shape):
    return np.asfortranarray(rng.standard_normal(shape).astype(np.float32))


@pytest.fixture(params=[0, 1], ids=["tiled", "direct"])
def path(request, pkg):
    lib = pkg.native_library()
    lib.pp_set_path(request.param)
    yield request.param
    lib.pp_set_path(0)


def _oracle_grad_dot(O, f0, phi, up, s):
    g = O.pull_grad(f0, phi, s)                     # (d1, 3, C[, B])
    if g.ndim == 5:
        return np.einsum("xyzkc,xyzc->xyzk", g, up.astype(np.float64))
    return np.einsum("xyzkcb,xyzcb->xyzkb", g, up.astype(np.float64))


def _oracle_hess_dot(O, f0, phi, up, s):
    h = O.pull_hess(f0, phi, s)                     # (d1, 3, 3, C)
    return np.einsum("xyzpqc,xyzqc->xyzp", h, up.astype(np.float64))


@pytest.mark.parametrize("deg,bnd,ext", [(1, 0, 0), (2, (0, 1, 2), 1), (3, 1, 1), (4, 2, 1), ((3, 1, 2), 1, 1)])
def test_pull_grad_dot(pkg, O, path, deg, bnd, ext):
    L = pkg.layout
    rng = np.random.default_rng(21)
    d0, d1 = (29, 25, 21), (26, 22, 17)
    f0, up = _f(rng, d0 + (2,)), _f(rng, d1 + (2,))
    phi = _phi(O, rng, d1, d0, 1.5)
    s, so = pkg.Settings(deg, bnd, ext), O.Sett.make(deg, bnd, ext)
    got = pkg.pull_grad_dot(L.from_numpy(f0), L.from_numpy(phi), L.from_numpy(up), s)
    assert tuple(got.shape) == phi.shape
    assert rel_err(L.to_numpy(got), _oracle_grad_dot(O, f0, phi, up, so)) <= 1e-4


@pytest.mark.parametrize("deg,bnd,ext", [(2, 1, 1), (3, (0, 1, 2), 0), (4, 0, 1)])
def test_pull_hess_dot(pkg, O, path, deg, bnd, ext):
    L = pkg.layout
    rng = np.random.default_rng(22)
    d0, d1 = (27, 23, 19), (24, 20, 16)
    f0, up = _f(rng, d0 + (2,)), _f(rng, d1 + (3, 2))
    phi = _phi(O, rng, d1, d0, 1.5)
    s, so = pkg.Settings(deg, bnd, ext), O.Sett.make(deg, bnd, ext)
    got = pkg.pull_hess_dot(L.from_numpy(f0), L.from_numpy(phi), L.from_numpy(up), s)
    assert rel_err(L.to_numpy(got), _oracle_hess_dot(O, f0, phi, up, so)) <= 1e-4


def _oracle_fused(O, f0, phi, g, s):
    r = O.pull(f0, phi, s) - g.astype(np.float64)
    loss = float(np.sum(r * r))
    d = np.asfortranarray((2 * r).astype(np.float32))
    df = O.push(d, phi, f0.shape[:3], s)
    gr = O.pull_grad(f0, phi, s)
    if r.ndim == 3:                                   # single channel without a channel axis
        return loss, df, gr * (2 * r)[..., None]
    dphi = np.einsum("xyzkc,xyzc->xyzk", gr, 2 * r)
    return loss, df, dphi


@pytest.mark.parametrize("deg,bnd,ext,nc", [(2, (0, 1, 2), 1, 1), (3, 1, 1, 2), (1, 0, 1, 3), (4, 2, 1, 1)])
def test_fused_step_vs_oracle(pkg, O, path, deg, bnd, ext, nc):
    L = pkg.layout
    rng = np.random.default_rng(31 + nc)
    d0, d1 = (33, 29, 23), (30, 27, 21)
    f0 = _f(rng, d0 + (nc,))
    phi = _phi(O, rng, d1, d0, 1.5)
    g = _f(rng, d1 + (nc,))
    s, so = pkg.Settings(deg, bnd, ext), O.Sett.make(deg, bnd, ext)
    loss, df, dphi = pkg.fused_step(L.from_numpy(f0), L.from_numpy(phi), L.from_numpy(g), s)
    ref_loss, ref_df, ref_dphi = _oracle_fused(O, f0, phi, g, so)
    assert abs(float(loss) - ref_loss) <= 1e-5 * abs(ref_loss)
    assert rel_err(L.to_numpy(df), ref_df) <= 1e-4
    assert rel_err(L.to_numpy(dphi), ref_dphi) <= 1e-4


def test_fused_step_batch_of_two(pkg, O, path):
    """Two channels and a batch of two: the loss sums over both, df and dphi are
    per batch element (the oracle runs each element on its own)."""
    L = pkg.layout
    rng = np.random.default_rng(47)
    d0, d1 = (31, 27, 22), (29, 26, 20)
    f0 = _f(rng, d0 + (2, 2))
    phi = np.asfortranarray(np.stack([_phi(O, rng, d1, d0, 1.5) for _ in range(2)], axis=-1))
    g = _f(rng, d1 + (2, 2))
    s, so = pkg.Settings(3, (0, 1, 2), 1), O.Sett.make(3, (0, 1, 2), 1)
    loss, df, dphi = pkg.fused_step(L.from_numpy(f0), L.from_numpy(phi), L.from_numpy(g), s)
    parts = [_oracle_fused(O, np.asfortranarray(f0[..., b]), np.asfortranarray(phi[..., b]),
                           np.asfortranarray(g[..., b]), so) for b in range(2)]
    ref_loss = sum(p[0] for p in parts)
    assert abs(float(loss) - ref_loss) <= 1e-5 * abs(ref_loss)
    assert rel_err(L.to_numpy(df), np.stack([p[1] for p in parts], axis=-1)) <= 1e-4
    assert rel_err(L.to_numpy(dphi), np.stack([p[2] for p in parts], axis=-1)) <= 1e-4


def test_fused_step_nan_and_reproducible(pkg, O, path):
    """ext = 0 voxels outside the band make the loss NaN and their dphi NaN; the loss
    is bit-identical from run to run (fixed-order reduction)."""
    L = pkg.layout
    rng = np.random.default_rng(5)
    d = (24, 20, 18)
    f0, g = _f(rng, d), _f(rng, d)
    phi = _phi(O, rng, d, d, 1.0)
    s = pkg.Settings(2, 1, 1)
    a = pkg.fused_step(L.from_numpy(f0), L.from_numpy(phi), L.from_numpy(g), s)
    b = pkg.fused_step(L.from_numpy(f0), L.from_numpy(phi), L.from_numpy(g), s)
    assert float(a[0]) == float(b[0])
    phi[0, 0, 0, 0] = -5.0
    loss, df, dphi = pkg.fused_step(L.from_numpy(f0), L.from_numpy(phi), L.from_numpy(g), pkg.Settings(2, 1, 0))
    ref_loss, ref_df, ref_dphi = _oracle_fused(O, f0, phi, g, O.Sett.make(2, 1, 0))
    assert np.isnan(float(loss)) and np.isnan(ref_loss)
    assert rel_err(L.to_numpy(dphi), ref_dphi) <= 1e-4
    assert rel_err(L.to_numpy(df), ref_df) <= 1e-4


def test_autograd_rules_match_fused(pkg, O, path):
    """loss = Σ (pull(f, ϕ) - g)² through the Pull rule equals the fused kernel's gradients;
    the Push and PullGrad rules agree with the oracle adjoints."""
    L = pkg.layout
    A = pkg.autograd
    rng = np.random.default_rng(41)
    d0, d1 = (26, 24, 20), (25, 22, 19)
    f0, g = _f(rng, d0 + (2,)), _f(rng, d1 + (2,))
    phi = _phi(O, rng, d1, d0, 1.2)
    s, so = pkg.Settings(3, (0, 1, 2), 1), O.Sett.make(3, (0, 1, 2), 1)
    tf, tp, tg = (L.from_numpy(a).requires_grad_(True) for a in (f0, phi, g))
    loss = ((A.pull(tf, tp, s) - tg.detach()) ** 2).sum()
    loss.backward()
    _, df, dphi = pkg.fused_step(tf.detach(), tp.detach(), tg.detach(), s)
    assert rel_err(L.to_numpy(tf.grad), L.to_numpy(df)) <= 1e-4
    assert rel_err(L.to_numpy(tp.grad), L.to_numpy(dphi)) <= 1e-4
    # push rule: d/df1 <push(f1), w> = pull(w); d/dphi = Σ f1 ∇pull(w)
    f1, w = _f(rng, d1 + (2,)), _f(rng, d0 + (2,))
    t1, tp2 = L.from_numpy(f1).requires_grad_(True), L.from_numpy(phi).requires_grad_(True)
    (A.push(t1, tp2, d0, s) * L.from_numpy(w)).sum().backward()
    assert rel_err(L.to_numpy(t1.grad), O.pull(w, phi, so)) <= 1e-4
    assert rel_err(L.to_numpy(tp2.grad), _oracle_grad_dot(O, w, phi, f1, so)) <= 1e-4
    # pull_grad rule: d/dphi <pull_grad(f), u> = Σ H u ; d/df = push_grad(u)
    u = _f(rng, d1 + (3, 2))
    tf3, tp3 = L.from_numpy(f0).requires_grad_(True), L.from_numpy(phi).requires_grad_(True)
    (A.pull_grad(tf3, tp3, s) * L.from_numpy(u)).sum().backward()
    assert rel_err(L.to_numpy(tp3.grad), _oracle_hess_dot(O, f0, phi, u, so)) <= 1e-4
    assert rel_err(L.to_numpy(tf3.grad), O.push_grad(u, phi, d0, so)) <= 1e-4


def test_fused_gradient_finite_differences(pkg, O, path):
    """Differentiable step (160x192x160-style settings: degree 2, bounds (0,1,2)) on a
    smaller volume: dphi against central differences of the FP64 loss at 64 random
    voxels (h = 1e-3 voxel, the actual float32 step used), df against differences of
    the FP64 loss in f at 16 random image voxels."""
    L = pkg.layout
    rng = np.random.default_rng(77)
    d = (40, 48, 40)
    import importlib
    W = importlib.import_module("pushpull_gb300.workloads")
    f0 = W.image(d, 3, fwhm=3.0)
    phi = _phi(O, rng, d, d, 1.5)
    g = np.asfortranarray(O.pull(f0, _phi(O, rng, d, d, 1.5), O.Sett.make(2, (0, 1, 2), 1)).astype(np.float32))
    s, so = pkg.Settings(2, (0, 1, 2), 1), O.Sett.make(2, (0, 1, 2), 1)
    loss, df, dphi = pkg.fused_step(L.from_numpy(f0), L.from_numpy(phi), L.from_numpy(g), s)
    dphi = L.to_numpy(dphi)
    ana, fd = [], []
    idx = rng.integers(0, [d[0], d[1], d[2]], size=(64, 3))
    for (i, j, k) in idx:
        for comp in range(3):
            p = phi[i, j, k, :].copy()
            x0 = p[comp]
            pp, pm = p.copy(), p.copy()
            pp[comp] = np.float32(x0 + np.float32(1e-3))
            pm[comp] = np.float32(x0 - np.float32(1e-3))
            lp = (O.pull_at(pp, f0, so) - float(g[i, j, k])) ** 2
            lm = (O.pull_at(pm, f0, so) - float(g[i, j, k])) ** 2
            fd.append((lp - lm) / (float(pp[comp]) - float(pm[comp])))
            ana.append(float(dphi[i, j, k, comp]))
    ana, fd = np.array(ana), np.array(fd)
    assert np.sum((ana - fd) ** 2) / np.sum(ana ** 2) < 1e-3
    # df: the loss is quadratic in f, so central differences are exact up to rounding
    dfn = L.to_numpy(df)
    r = O.pull(f0, phi, so) - g
    base = float(np.sum(r * r))
    assert abs(float(loss) - base) <= 1e-5 * base
    for (i, j, k) in rng.integers(0, [d[0], d[1], d[2]], size=(16, 3)):
        fp = f0.copy(order="F")
        h = 1e-2
        fp[i, j, k] = f0[i, j, k] + np.float32(h)
        hp = float(fp[i, j, k]) - float(f0[i, j, k])
        lp = float(np.sum((O.pull(fp, phi, so) - g) ** 2))
        fp[i, j, k] = f0[i, j, k] - np.float32(h)
        hm = float(f0[i, j, k]) - float(fp[i, j, k])
        lm = float(np.sum((O.pull(fp, phi, so) - g) ** 2))
        fdv = (lp - lm) / (hp + hm)
        assert abs(fdv - float(dfn[i, j, k])) <= 1e-3 * max(1.0, abs(fdv))
