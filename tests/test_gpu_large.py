"""Maximum sizes: an image of more than 2^31 voxels (8.6 GB) takes the 64-bit
index kernels.  Samples scattered over the whole image are pulled and checked
against the FP64 oracle run on a host copy of the image; push through the same
samples is checked by the adjoint identity (sums in float64 on the device)."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


def test_image_beyond_2_31_voxels(pkg, O):
    L = pkg.layout
    d0 = (1312, 1312, 1250)                        # 2.15e9 voxels > 2^31
    assert np.prod(d0) > 2 ** 31
    d1 = (40, 36, 32)
    free, _ = torch.cuda.mem_get_info()
    if free < 40 * 2 ** 30:
        pytest.skip("needs 40 GB of free device memory")
    g = torch.Generator(device="cuda").manual_seed(5)
    f0 = L.empty(d0)
    L.flat(f0).uniform_(generator=g)
    rng = np.random.default_rng(6)
    phi_np = np.empty(d1 + (3,), dtype=np.float32, order="F")
    for k in range(3):                             # samples spread over the whole image
        phi_np[..., k] = rng.uniform(-2.0, d0[k] + 2.0, d1).astype(np.float32)
    phi = L.from_numpy(phi_np)
    for deg, bnd in [(1, 0), (3, 1), (2, 2)]:
        s, so = pkg.Settings(deg, bnd, 1), O.Sett.make(deg, bnd, 1)
        got = L.to_numpy(pkg.pull(f0, phi, s))
        # the oracle reads the image from host memory: 8.6 GB, copied once
        if deg == 1:
            f0_host = L.to_numpy(f0)
        ref = O.pull(f0_host, phi_np, so)
        assert rel_err(got, ref) <= 1e-5, (deg, bnd)
        a = L.from_numpy(rng.standard_normal(d1).astype(np.float32))
        pushed = pkg.push(a, phi, d0, s)
        lhs = sum(float(torch.dot(L.flat(pushed)[i:i + 2 ** 28].double(), L.flat(f0)[i:i + 2 ** 28].double()))
                  for i in range(0, int(np.prod(d0)), 2 ** 28))
        rhs = float((a.double() * pkg.pull(f0, phi, s).double()).sum())
        assert abs(lhs - rhs) <= 1e-5 * abs(rhs), (deg, bnd, lhs, rhs)
        del pushed
        torch.cuda.empty_cache()
