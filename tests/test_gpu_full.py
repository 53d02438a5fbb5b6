"""Full-size cases of the benchmark workloads, against the FP64 oracle and through
size-independent properties.

* 192^3 cubic DCT-II (the pull+push benchmark): pull within 1e-5 and push within
  1e-4 of the FP64 oracle (norm-wise relative); adjoint identity
  |<f1, pull(f2)> - <push(f1), f2>| <= 1e-5 relative (sums in float64).
* 160x192x160 quadratic, bounds (0,1,2) (the differentiable step): fused loss
  within 1e-5, df and dphi within 1e-4 of the FP64 oracle.
"""
from __future__ import annotations

import importlib

import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


@pytest.fixture(scope="module")
def W(pkg):
    return importlib.import_module("pushpull_gb300.workloads")


def test_c2_pull_push_vs_oracle_and_adjoint(pkg, O, W):
    L = pkg.layout
    w = W.config2()
    s, so = pkg.Settings(w.deg, w.bnd, w.ext), O.Sett.make(w.deg, w.bnd, w.ext)
    f0, phi = L.from_numpy(w.f0), L.from_numpy(w.phi)
    f1 = pkg.pull(f0, phi, s)
    back = pkg.push(f1, phi, w.f0.shape[:3], s)
    torch.cuda.synchronize()
    f1n = L.to_numpy(f1)
    assert rel_err(f1n, O.pull(w.f0, w.phi, so)) <= 1e-5
    assert rel_err(L.to_numpy(back), O.push(f1n, w.phi, w.f0.shape[:3], so)) <= 1e-4
    rng = np.random.default_rng(0)
    a = L.from_numpy(np.asfortranarray(rng.standard_normal(w.phi.shape[:3]).astype(np.float32)))
    b = L.from_numpy(np.asfortranarray(rng.standard_normal(w.f0.shape[:3]).astype(np.float32)))
    lhs = float((a.double() * pkg.pull(b, phi, s).double()).sum())
    rhs = float((pkg.push(a, phi, w.f0.shape[:3], s).double() * b.double()).sum())
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)


def test_c3_fused_step_vs_oracle(pkg, O, W):
    L = pkg.layout
    w = W.config3()
    s, so = pkg.Settings(w.deg, w.bnd, w.ext), O.Sett.make(w.deg, w.bnd, w.ext)
    g = O.pull(w.f0, w.extra["phi2"], so).astype(np.float32)
    g = np.asfortranarray(g)
    loss, df, dphi = pkg.fused_step(L.from_numpy(w.f0), L.from_numpy(w.phi), L.from_numpy(g), s)
    r = O.pull(w.f0, w.phi, so) - g
    ref_loss = float(np.sum(r * r))
    assert abs(float(loss) - ref_loss) <= 1e-5 * ref_loss
    d = np.asfortranarray((2 * r).astype(np.float32))
    assert rel_err(L.to_numpy(df), O.push(d, w.phi, w.f0.shape[:3], so)) <= 1e-4
    ref_dphi = O.pull_grad(w.f0, w.phi, so) * (2 * r)[..., None]
    assert rel_err(L.to_numpy(dphi), ref_dphi) <= 1e-4


def test_c5_contention_push_vs_oracle(pkg, O, W):
    """Many-to-one scatter (0.25x contraction + FWHM-12 field of +-3 vox, cubic,
    DCT-II, 3 channels): push and push_grad within 1e-4 of the FP64 oracle at
    128^3, and at the full 256^3 the adjoint identity <push(a), b> = <a, pull(b)>
    within 1e-5 (sums in float64)."""
    L = pkg.layout
    s, so = pkg.Settings(3, 1, 1), O.Sett.make(3, 1, 1)
    d = (128, 128, 128)
    f1 = np.asfortranarray(W.image(d, 61, channels=3))
    g1 = np.asfortranarray(np.random.default_rng(62).standard_normal(d + (3, 3)).astype(np.float32))
    phi = W.deformation(d, 63, 12.0, 3.0, contraction=0.25)
    got = L.to_numpy(pkg.push(L.from_numpy(f1), L.from_numpy(phi), d, s))
    assert rel_err(got, O.push(f1, phi, d, so)) <= 1e-4
    got = L.to_numpy(pkg.push_grad(L.from_numpy(g1), L.from_numpy(phi), d, s))
    assert rel_err(got, O.push_grad(g1, phi, d, so)) <= 1e-4
    d = (256, 256, 256)
    a = W.image_gpu(d, 64, channels=3)
    b = W.image_gpu(d, 65, channels=3)
    phi = W.deformation_gpu(d, 66, 12.0, 3.0, contraction=0.25)
    lhs = float((pkg.push(a, phi, d, s).double() * b.double()).sum())
    rhs = float((a.double() * pkg.pull(b, phi, s).double()).sum())
    assert abs(lhs - rhs) <= 1e-5 * abs(rhs)
