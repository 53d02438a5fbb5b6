"""Compositions (compose, Exp, the graph-captured ExpPlan) and push with a count
image, against the FP64 oracle.

compose is one pull, so it is held to the pull tolerance (1e-5, norm-wise
relative).  Exp chains eight of them; the oracle runs the same recursion (FP64
pulls, positions rounded to float32 as the device sees them) and the resulting
positions must agree within 1e-5 (eight compositions amplify float32-level
perturbations of u about sevenfold).  push_count: both outputs within 1e-4 of the oracle's push of the
values and of ones, with non-finite values skipped in both."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

BND = [(2, 1, 1), (1, 2, 1), (1, 1, 2)]


def _field(rng, d, amp):
    from scipy.ndimage import gaussian_filter
    u = np.stack([gaussian_filter(rng.standard_normal(d), 2.0, mode="wrap") for _ in range(3)], axis=-1)
    u *= amp / np.abs(u).max()
    return np.asfortranarray(u.astype(np.float32))


def test_compose_vs_oracle(pkg, O):
    L = pkg.layout
    rng = np.random.default_rng(41)
    d = (24, 20, 16)
    Id = O.identity(d)
    phi = np.asfortranarray(Id + _field(rng, d, 2.0))
    theta = np.asfortranarray(Id + _field(rng, d, 3.0))
    got = L.to_numpy(pkg.compose(L.from_numpy(phi), L.from_numpy(theta)))
    ref = O.pull(phi, theta, O.Sett.make(1, BND, 1))
    assert rel_err(got, ref) <= 1e-5


def test_exp_vs_oracle_and_plan(pkg, O):
    L = pkg.layout
    rng = np.random.default_rng(42)
    d = (20, 18, 14)
    v = _field(rng, d, 4.0)
    Id = O.identity(d).astype(np.float32)
    so = O.Sett.make(1, BND, 1)
    u = (v / np.float32(256)).astype(np.float32)
    for _ in range(8):
        u = np.asfortranarray(O.pull(u, np.asfortranarray((Id + u).astype(np.float32)), so).astype(np.float32))
    ref = u + Id
    got = L.to_numpy(pkg.Exp(L.from_numpy(v)))
    assert rel_err(got, ref) <= 1e-5
    plan = pkg.ExpPlan(d)
    out = L.to_numpy(plan(L.from_numpy(v)))
    assert np.array_equal(out, got)               # the same kernels in the same order
    v2 = _field(rng, d, 2.0)                     # the plan is reusable with new inputs
    out2 = L.to_numpy(plan(L.from_numpy(v2)))
    assert np.array_equal(out2, L.to_numpy(pkg.Exp(L.from_numpy(v2))))


@pytest.mark.parametrize("deg,bnd", [(1, 2), (2, (0, 1, 2)), (3, 1)])
def test_push_count_vs_oracle(pkg, O, deg, bnd):
    L = pkg.layout
    rng = np.random.default_rng(43)
    d0, d1 = (22, 19, 15), (20, 17, 13)
    phi = O.identity(d1).astype(np.float64)
    for k in range(3):
        phi[..., k] = 1 + (phi[..., k] - 1) * (d0[k] - 1) / (d1[k] - 1)
    phi = np.asfortranarray((phi + 1.5 * rng.standard_normal(phi.shape)).astype(np.float32))
    f1 = np.asfortranarray(rng.standard_normal(d1 + (2,)).astype(np.float32))
    f1[3, 4, 5, 0] = np.nan
    f1[7, 1, 2, 1] = np.inf
    s, so = pkg.Settings(deg, bnd, 1), O.Sett.make(deg, bnd, 1)
    f0, c0 = pkg.push_count(L.from_numpy(f1), L.from_numpy(phi), d0, s)
    ones = np.where(np.isfinite(f1), np.float32(1), np.float32(np.nan)).astype(np.float32)
    assert rel_err(L.to_numpy(f0), O.push(f1, phi, d0, so)) <= 1e-4
    assert rel_err(L.to_numpy(c0), O.push(np.asfortranarray(ones), phi, d0, so)) <= 1e-4
    # accumulate adds into both outputs
    f0b, c0b = pkg.push_count(L.from_numpy(f1), L.from_numpy(phi), d0, s, out=f0.clone(), count=c0.clone(),
                              accumulate=True)
    assert rel_err(L.to_numpy(c0b), 2 * L.to_numpy(c0)) <= 1e-5
