"""pp_fused_step_noalloc, the fused step whose scratch lives in a fixed array
inside the library, for callers that cannot let a library allocate device
memory (their own allocator already holds the device's memory, or their request
path forbids allocation).

Called through the C ABI and compared with pp_fused_step on the same inputs, on
two calls in a row with different inputs (the shared array keeps the previous
call's contents), on both kernel families; sizes beyond the fixed scratch are
refused before anything is written.  This file is collected last on purpose.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu

PP_ERR_TOO_LARGE = 9


def _run(lib, name, f0, phi, g, sett, nc, nb):
    from pushpull_gb300 import _native, layout as L
    loss = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    df = L.empty(tuple(f0.shape), device="cuda")
    dphi = L.empty(tuple(phi.shape[:3]) + (3,) + ((nb,) if nb > 1 else ()), device="cuda")
    rc = getattr(lib, name)(loss.data_ptr(), df.data_ptr(), dphi.data_ptr(), f0.data_ptr(), phi.data_ptr(),
                            g.data_ptr(), _native.u64x3(f0.shape[:3]), _native.u64x3(phi.shape[:3]), nc, nb,
                            sett.bnd_array(), sett.nbnd, _native.i32x3(sett.deg), sett.ext, 0,
                            torch.cuda.current_stream().cuda_stream)
    return rc, loss, df, dphi


def _inputs(pkg, O, seed, d0, d1, nc, scale, nb=1):
    L = pkg.layout
    rng = np.random.default_rng(seed)
    cb = ((nc,) if nc > 1 or nb > 1 else ()) + ((nb,) if nb > 1 else ())
    f0 = scale * rng.standard_normal(d0 + cb).astype(np.float32)
    phis = []
    for _ in range(nb):
        phi = O.identity(d1).astype(np.float64)
        for k in range(3):
            phi[..., k] = 1 + (phi[..., k] - 1) * (d0[k] - 1) / max(d1[k] - 1, 1)
        phis.append((phi + 1.5 * rng.standard_normal(phi.shape)).astype(np.float32))
    phi = np.stack(phis, axis=-1) if nb > 1 else phis[0]
    g = scale * rng.standard_normal(d1 + cb).astype(np.float32)
    return tuple(L.from_numpy(np.asfortranarray(a)) for a in (f0, phi, g))


@pytest.mark.parametrize("path", [0, 1])
@pytest.mark.parametrize("nb", [1, 2])
def test_noalloc_matches_fused_step_two_calls(pkg, O, path, nb):
    """Two calls in a row (the second with different inputs); with nb = 2 the
    per-(channel, batch) plane maxima and the per-batch loss partials are
    compared for values as well."""
    lib = pkg.native_library()
    assert lib.pp_set_path(path) == 0
    try:
        sett = pkg.Settings(2, (0, 1, 2), 1)
        for call, (seed, scale) in enumerate([(1, 100.0), (2, 1.0)]):
            f0, phi, g = _inputs(pkg, O, seed + 10 * nb, (40, 36, 30), (38, 34, 28), 2, scale, nb)
            rc, loss, df, dphi = _run(lib, "pp_fused_step_noalloc", f0, phi, g, sett, 2, nb)
            assert rc == 0, lib.pp_last_error()
            rc, rloss, rdf, rdphi = _run(lib, "pp_fused_step", f0, phi, g, sett, 2, nb)
            assert rc == 0, lib.pp_last_error()
            torch.cuda.synchronize()
            a, b = float(loss), float(rloss)
            assert np.isfinite(a) and abs(a - b) <= 1e-5 * abs(b), (call, a, b)
            assert rel_err(pkg.layout.to_numpy(df), pkg.layout.to_numpy(rdf)) <= 1e-4
            assert rel_err(pkg.layout.to_numpy(dphi), pkg.layout.to_numpy(rdphi)) <= 1e-4
        assert lib.pp_device_status(1) == 0
    finally:
        lib.pp_set_path(0)


def test_noalloc_refuses_sizes_beyond_its_scratch(pkg, O):
    """nc*nb above the plane limit, and (per-voxel kernels) more loss partials
    than the array holds: PP_ERR_TOO_LARGE, outputs untouched."""
    from pushpull_gb300 import _native
    lib = pkg.native_library()
    L = pkg.layout
    sett = pkg.Settings(1, 1, 1)
    nb = 4100
    f0 = L.empty((2, 2, 2, 1, nb), device="cuda").fill_(1.0)
    phi = L.empty((2, 2, 2, 3, nb), device="cuda").fill_(1.0)
    g = L.empty((2, 2, 2, 1, nb), device="cuda").fill_(0.0)
    loss = torch.full((1,), 7.0, dtype=torch.float64, device="cuda")
    df = L.empty(tuple(f0.shape), device="cuda").fill_(3.0)
    dphi = L.empty((2, 2, 2, 3, nb), device="cuda").fill_(3.0)
    rc = lib.pp_fused_step_noalloc(loss.data_ptr(), df.data_ptr(), dphi.data_ptr(), f0.data_ptr(), phi.data_ptr(),
                                   g.data_ptr(), _native.u64x3((2, 2, 2)), _native.u64x3((2, 2, 2)), 1, nb,
                                   sett.bnd_array(), sett.nbnd, _native.i32x3(sett.deg), sett.ext, 0,
                                   torch.cuda.current_stream().cuda_stream)
    assert rc == PP_ERR_TOO_LARGE and b"planes" in lib.pp_last_error()
    torch.cuda.synchronize()
    assert float(loss) == 7.0 and bool((df == 3.0).all())
    assert lib.pp_set_path(1) == 0
    try:
        d, nb = (72, 72, 72), 8
        f0 = L.empty(d + (1, nb), device="cuda").fill_(1.0)
        phi = L.empty(d + (3, nb), device="cuda").fill_(1.0)
        g = L.empty(d + (1, nb), device="cuda").fill_(0.0)
        df = L.empty(tuple(f0.shape), device="cuda").fill_(3.0)
        dphi = L.empty(d + (3, nb), device="cuda")
        rc = lib.pp_fused_step_noalloc(loss.data_ptr(), df.data_ptr(), dphi.data_ptr(), f0.data_ptr(),
                                       phi.data_ptr(), g.data_ptr(), _native.u64x3(d), _native.u64x3(d), 1, nb,
                                       sett.bnd_array(), sett.nbnd, _native.i32x3(sett.deg), sett.ext, 0,
                                       torch.cuda.current_stream().cuda_stream)
        assert rc == PP_ERR_TOO_LARGE and b"partials" in lib.pp_last_error()
        torch.cuda.synchronize()
        assert bool((df == 3.0).all())
    finally:
        lib.pp_set_path(0)
