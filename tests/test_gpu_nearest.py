"""The nearest-neighbour pull kernel (degree 0: four sample voxels per thread,
16-byte deformation loads, the next group's deformation in flight while this
group gathers) against the FP64 oracle.  A degree-0 pull copies image values
(weights of one), so the results must equal the oracle's exactly:

* taps inside the image (lean path) and folded ones (every bound, positions
  several periods outside the image: the general path);
* NaN and infinite positions, ext = 0 with positions outside the band;
* several channels with per-channel bounds, a batch of two;
* pull_grad (all zeros at degree 0, NaN where the position is invalid);
* sample counts that are not a multiple of 4 (the one-voxel kernel) give the
  same values as the oracle too.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _phi(O, rng, d1, d0, sigma, nb):
    out = []
    for _ in range(nb):
        p = O.identity(d1).astype(np.float64)
        for k in range(3):
            p[..., k] = 1 + (p[..., k] - 1) * (d0[k] - 1) / max(d1[k] - 1, 1)
        out.append(p + sigma * rng.standard_normal(p.shape))
    return np.asfortranarray(np.stack(out, axis=-1).astype(np.float32))


def _check(pkg, O, f0, phi, bnd, ext):
    L = pkg.layout
    s, so = pkg.Settings(0, bnd, ext), O.Sett.make(0, bnd, ext)
    got = L.to_numpy(pkg.pull(L.from_numpy(f0), L.from_numpy(phi), s))
    gotg = L.to_numpy(pkg.pull_grad(L.from_numpy(f0), L.from_numpy(phi), s))
    assert pkg.native_library().pp_device_status(1) == 0
    nb = phi.shape[-1]
    for b in range(nb):
        fb, pb = np.asfortranarray(f0[..., b]), np.asfortranarray(phi[..., b])
        ref = O.pull(fb, pb, so, threads=8).astype(np.float32)
        refg = O.pull_grad(fb, pb, so, threads=8).astype(np.float32)
        assert np.array_equal(got[..., b], ref, equal_nan=True), b
        assert np.array_equal(gotg[..., b], refg, equal_nan=True), b


@pytest.mark.parametrize("d1", [(32, 24, 20), (21, 19, 13)], ids=["n1 % 4 == 0", "n1 % 4 != 0"])
def test_nearest_inside_folded_and_invalid(pkg, O, d1):
    rng = np.random.default_rng(900 + d1[0])
    d0 = (29, 23, 17)
    f0 = np.asfortranarray(rng.standard_normal(d0 + (3, 2)).astype(np.float32))
    phi = _phi(O, rng, d1, d0, 3.0, nb=2)
    flat = phi.reshape(-1, order="F")
    idx = rng.choice(flat.size, 60, replace=False)
    flat[idx[:10]] = np.nan
    flat[idx[10:20]] = np.inf
    flat[idx[20:40]] = rng.uniform(-200, 200, 20).astype(np.float32)   # several periods outside
    flat[idx[40:]] = rng.uniform(-6, 0, 20).astype(np.float32)          # just below the first voxel
    _check(pkg, O, f0, phi, [(0, 1, 2), (1, 1, 1), (2, 0, 1)], 1)
    _check(pkg, O, f0, phi, [(2, 2, 2), (0, 0, 0), (1, 2, 0)], 0)
