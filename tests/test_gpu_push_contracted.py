"""Push through contracting deformations: the contracted-tile scatter (one voxel
per warp step, per-lane register accumulation along runs of voxels, all
channels of a group in one walk) against the FP64 oracle, channel by channel:

* more channels than one walk takes (two groups), per-channel boundary triples;
* an all-zero channel, a channel with non-finite values (skipped), and
  channels whose scale bound leaves the fixed-point range (1e30 and 1e-30:
  float accumulation instead);
* quadratic and cubic, ext = 0 with voxels outside the band, batches;
* the tiled path against the per-voxel kernels on the same inputs.
Tolerance 1e-4 (norm-wise relative, per channel)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _phi(O, rng, d, contraction, sigma, nb=1):
    out = []
    c = 0.5 * (np.array(d, dtype=np.float64) + 1)
    for _ in range(nb):
        p = O.identity(d).astype(np.float64)
        for k in range(3):
            p[..., k] = c[k] + contraction * (p[..., k] - c[k])
        out.append(p + sigma * rng.standard_normal(p.shape))
    a = np.stack(out, axis=-1) if nb > 1 else out[0]
    return np.asfortranarray(a.astype(np.float32))


def _values(rng, d, nb):
    nc = 6
    f = rng.standard_normal(d + (nc, nb)).astype(np.float64)
    f[..., 1, :] = 0.0                                   # nothing to push
    f[..., 2, :][rng.random(d + (nb,)) < 0.02] = np.nan   # skipped values
    f[..., 3, :] *= 1e30                                 # scale bound beyond the fixed-point range
    f[..., 4, :] *= 1e-30                                # and below it
    f[..., 5, :] = -np.abs(f[..., 5, :])
    return np.asfortranarray(f.astype(np.float32))


@pytest.mark.parametrize("deg,ext", [(3, 1), (2, 1), (3, 0)])
def test_contracted_push_vs_oracle(pkg, O, deg, ext):
    L = pkg.layout
    rng = np.random.default_rng(500 + deg + 10 * ext)
    d, nb = (48, 44, 40), 2
    phi = _phi(O, rng, d, 0.2, 0.4, nb)
    f1 = _values(rng, d, nb)
    bnd = [(1, 1, 1), (0, 1, 2), (2, 2, 2), (1, 0, 1), (0, 0, 0), (2, 1, 0)]
    s, so = pkg.Settings(deg, bnd, ext), O.Sett.make(deg, bnd, ext)
    got = L.to_numpy(pkg.push(L.from_numpy(f1), L.from_numpy(phi), d, s))
    assert pkg.native_library().pp_device_status(1) == 0
    ref = O.push(f1, phi, d, so)
    for b in range(nb):
        assert not np.any(got[..., 1, b]), "an all-zero channel pushes zeros"
        for c in (0, 2, 3, 4, 5):
            assert np.isfinite(got[..., c, b]).all()
            assert rel_err(got[..., c, b], ref[..., c, b]) <= 1e-4, (c, b)
    # the per-voxel kernels on the same inputs
    lib = pkg.native_library()
    assert lib.pp_set_path(1) == 0
    try:
        direct = L.to_numpy(pkg.push(L.from_numpy(f1), L.from_numpy(phi), d, s))
    finally:
        lib.pp_set_path(0)
    for c in (0, 2, 3, 4, 5):
        assert rel_err(got[..., c, :], direct[..., c, :]) <= 1e-4, c


@pytest.mark.parametrize("deg", [3, 2])
def test_contracted_push_grad_vs_oracle(pkg, O, deg):
    """push_grad on contracted tiles (records of v0 dw_x, v1 w_x, v2 w_x and the
    y and z weights and derivatives), per-channel bounds, a channel of zeros and
    one beyond the fixed-point range, against FP64 and the per-voxel kernels."""
    L = pkg.layout
    rng = np.random.default_rng(700 + deg)
    d, nb, nc = (44, 40, 36), 2, 3
    phi = _phi(O, rng, d, 0.2, 0.4, nb)
    g = rng.standard_normal(d + (3, nc, nb))
    g[..., 1, :] = 0.0
    g[..., 2, :] *= 1e30
    g = np.asfortranarray(g.astype(np.float32))
    bnd = [(1, 1, 1), (0, 1, 2), (2, 0, 1)]
    s, so = pkg.Settings(deg, bnd, 1), O.Sett.make(deg, bnd, 1)
    got = L.to_numpy(pkg.push_grad(L.from_numpy(g), L.from_numpy(phi), d, s))
    lib = pkg.native_library()
    assert lib.pp_device_status(1) == 0
    ref = O.push_grad(g, phi, d, so)
    for b in range(nb):
        assert not np.any(got[..., 1, b])
        for c in (0, 2):
            assert np.isfinite(got[..., c, b]).all()
            assert rel_err(got[..., c, b], ref[..., c, b]) <= 1e-4, (c, b)
    assert lib.pp_set_path(1) == 0
    try:
        direct = L.to_numpy(pkg.push_grad(L.from_numpy(g), L.from_numpy(phi), d, s))
    finally:
        lib.pp_set_path(0)
    for c in (0, 2):
        assert rel_err(got[..., c, :], direct[..., c, :]) <= 1e-4, c
