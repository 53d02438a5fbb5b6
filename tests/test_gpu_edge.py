"""Edge cases through the native path: empty sample grids (every op is a no-op
that still zeroes a non-accumulating push output, and the fused loss is 0) and
size-1 dimensions on the tiled kernels' fallback to the per-voxel ones."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu


def test_empty_sample_grid(pkg):
    L = pkg.layout
    s = pkg.Settings(3, 1, 1)
    f0 = L.empty((8, 8, 8))
    L.flat(f0).uniform_()
    phi = L.empty((0, 4, 4, 3))
    assert tuple(pkg.pull(f0, phi, s).shape) == (0, 4, 4)
    assert tuple(pkg.pull_grad(f0, phi, s).shape) == (0, 4, 4, 3)
    f1 = L.empty((0, 4, 4))
    out = L.empty((8, 8, 8))
    L.flat(out).fill_(5.0)
    back = pkg.push(f1, phi, (8, 8, 8), s, out=out, accumulate=False)
    assert float(back.abs().sum()) == 0.0
    out.fill_(5.0)
    back = pkg.push(f1, phi, (8, 8, 8), s, out=out, accumulate=True)
    assert bool((back == 5.0).all())
    loss, df, dphi = pkg.fused_step(f0, phi, f1, s)
    torch.cuda.synchronize()
    assert float(loss) == 0.0 and float(df.abs().sum()) == 0.0


def test_size_one_dimensions(pkg, O):
    L = pkg.layout
    rng = np.random.default_rng(51)
    d0, d1 = (1, 30, 20), (1, 28, 16)
    f0 = np.asfortranarray(rng.standard_normal(d0).astype(np.float32))
    phi = O.identity(d1).astype(np.float64)
    phi[..., 1:] += 1.5 * rng.standard_normal(phi[..., 1:].shape)
    phi = np.asfortranarray(phi.astype(np.float32))
    f1 = np.asfortranarray(rng.standard_normal(d1).astype(np.float32))
    for deg, bnd in [(1, 0), (3, 1), (2, 2)]:
        s, so = pkg.Settings(deg, bnd, 1), O.Sett.make(deg, bnd, 1)
        assert rel_err(L.to_numpy(pkg.pull(L.from_numpy(f0), L.from_numpy(phi), s)), O.pull(f0, phi, so)) <= 1e-5
        assert rel_err(L.to_numpy(pkg.push(L.from_numpy(f1), L.from_numpy(phi), d0, s)),
                       O.push(f1, phi, d0, so)) <= 1e-4
