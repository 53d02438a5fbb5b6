"""The warp-specialised pull kernels (8 x 8 x 30 tiles; fifteen consumer warps
evaluate while one producer warp streams the deformation and stages interior
boxes) against the FP64 oracle, on every path they take, for pull, pull_grad,
pull_hess and the two cotangent contractions (pull_grad_dot, pull_hess_dot):

* interior boxes staged by one TMA copy of the fixed window;
* boundary boxes gathered by the consumers with folding and DST-II signs, with
  16-byte row chunks (image x extent a multiple of 4) and without (odd x
  extent, so no TMA window either);
* boxes too large for a buffer (strong local expansion): per-voxel fallback;
* non-finite deformations, far-out coordinates, ext = 0 bands, several
  channels with per-channel boundaries, batches, every degree;
* a deformation whose x extent rules out TMA: the call falls back to the
  block-synchronous kernels.
Tolerances: pull 1e-5, pull_grad 1e-4 (norm-wise), NaN masks identical."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture
def ws(pkg):
    lib = pkg.native_library()
    saved = {}
    for op in range(6):
        for d in range(5):
            v = [C.c_int() for _ in range(4)]
            assert lib.pp_get_tile(op, d, *[C.byref(x) for x in v]) == 0
            saved[(op, d)] = [x.value for x in v]
    for op in (0, 1, 2):
        assert lib.pp_set_tile(op, -1, 3, 3, 4, 15360) == 0, lib.pp_last_error()
    yield lib
    for (op, d), v in saved.items():
        lib.pp_set_tile(op, d, *v)
    lib.pp_set_path(0)


def _phi(O, rng, d1, d0, sigma, nb=1):
    out = []
    for _ in range(nb):
        p = O.identity(d1).astype(np.float64)
        for k in range(3):
            p[..., k] = 1 + (p[..., k] - 1) * (d0[k] - 1) / max(d1[k] - 1, 1)
        out.append(p + sigma * rng.standard_normal(p.shape))
    a = np.stack(out, axis=-1) if nb > 1 else out[0]
    return np.asfortranarray(a.astype(np.float32))


def _check(pkg, O, f0, phi, deg, bnd, ext):
    L = pkg.layout
    s, so = pkg.Settings(deg, bnd, ext), O.Sett.make(deg, bnd, ext)
    tf0, tphi = L.from_numpy(f0), L.from_numpy(phi)
    got = L.to_numpy(pkg.pull(tf0, tphi, s))
    gotg = L.to_numpy(pkg.pull_grad(tf0, tphi, s))
    torch.cuda.synchronize()
    e1 = rel_err(got, O.pull(f0, phi, so, threads=8))
    e2 = rel_err(gotg, O.pull_grad(f0, phi, so, threads=8))
    assert e1 <= 1e-5 and e2 <= 1e-4, (deg, bnd, ext, e1, e2)
    assert pkg.native_library().pp_device_status(1) == 0


@pytest.mark.parametrize("deg", [0, 1, 2, 3, 4])
def test_ws_interior_and_boundary_boxes(pkg, O, ws, deg):
    rng = np.random.default_rng(100 + deg)
    d0 = d1 = (40, 36, 44)
    f0 = np.asfortranarray(rng.standard_normal(d0 + (2, 2)).astype(np.float32))
    phi = _phi(O, rng, d1, d0, 1.5, nb=2)
    _check(pkg, O, f0, phi, deg, [(0, 1, 2), (2, 2, 2)], 1)
    _check(pkg, O, f0, phi, deg, [(1, 1, 1), (0, 0, 0)], 0)


@pytest.mark.parametrize("deg", [1, 3])
def test_ws_gathered_boxes_without_vector_rows(pkg, O, ws, deg):
    """Image x extent 37: no TMA window and no 16-byte rows; every box gathered per element."""
    rng = np.random.default_rng(200 + deg)
    d0, d1 = (37, 29, 35), (32, 24, 40)
    f0 = np.asfortranarray(rng.standard_normal(d0).astype(np.float32))
    phi = _phi(O, rng, d1, d0, 2.0)
    _check(pkg, O, f0, phi, deg, (2, 1, 0), 1)


def test_ws_large_boxes_take_the_per_voxel_path(pkg, O, ws):
    """A 32^3 sample grid spread over a 96^3 image (3x expansion): tile boxes exceed a buffer."""
    rng = np.random.default_rng(300)
    d0, d1 = (96, 96, 96), (32, 32, 32)
    f0 = np.asfortranarray(rng.standard_normal(d0).astype(np.float32))
    phi = _phi(O, rng, d1, d0, 0.5)
    for deg in (2, 3):
        _check(pkg, O, f0, phi, deg, 1, 1)


def test_ws_nonfinite_and_out_of_band(pkg, O, ws):
    rng = np.random.default_rng(400)
    d0 = d1 = (32, 24, 32)
    f0 = np.asfortranarray(rng.standard_normal(d0 + (3,)).astype(np.float32))
    phi = _phi(O, rng, d1, d0, 2.5)
    flat = phi.reshape(-1, order="F")
    idx = rng.choice(flat.size, 40, replace=False)
    flat[idx[:15]] = np.nan
    flat[idx[15:25]] = np.inf
    flat[idx[25:]] = 1e6                               # far out: those tiles take the per-voxel path
    for deg in (1, 3):
        _check(pkg, O, f0, phi, deg, [(0, 1, 2), (1, 1, 1), (2, 0, 1)], 0)
        _check(pkg, O, f0, phi, deg, 1, 1)


def test_ws_falls_back_when_tma_cannot_stream_phi(pkg, O, ws):
    """Sample grid x extent 30 (rows not 16-byte multiples): the block-synchronous kernels run."""
    rng = np.random.default_rng(500)
    d0, d1 = (36, 28, 36), (30, 28, 36)
    f0 = np.asfortranarray(rng.standard_normal(d0).astype(np.float32))
    phi = _phi(O, rng, d1, d0, 1.0)
    _check(pkg, O, f0, phi, 3, 1, 1)


@pytest.mark.parametrize("z", [14, 15, 16, 31, 61])
def test_ws_sample_depths_around_the_tile(pkg, O, ws, z):
    """Sample grids 14..61 deep against 30-deep tiles: 15 or more take the
    warp-specialised kernels (partial last tiles), 14 the block-synchronous ones;
    pull and pull_grad agree with FP64 either way."""
    rng = np.random.default_rng(600 + z)
    d0, d1 = (40, 32, z + 4), (40, 32, z)
    f0 = np.asfortranarray(rng.standard_normal(d0 + (2, 2)).astype(np.float32))
    phi = _phi(O, rng, d1, d0, 1.2, nb=2)
    _check(pkg, O, f0, phi, 3, [(1, 1, 1), (2, 0, 1)], 1)
    _check(pkg, O, f0, phi, 2, 0, 0)


@pytest.mark.parametrize("deg", [1, 2, 3, 4])
def test_ws_hessian_and_dot_ops(pkg, O, ws, deg):
    """pull_hess, pull_grad_dot and pull_hess_dot on the warp-specialised kernels
    (the dot ops sum their channels in the output array): two channels with
    per-channel bounds, a batch of two, interior and boundary boxes, against FP64
    and against the per-voxel kernels on the same inputs."""
    L = pkg.layout
    lib = pkg.native_library()
    rng = np.random.default_rng(800 + deg)
    d0 = d1 = (40, 36, 44)
    nb = 2
    f0 = np.asfortranarray(rng.standard_normal(d0 + (2, nb)).astype(np.float32))
    phi = _phi(O, rng, d1, d0, 1.5, nb=nb)
    ug = np.asfortranarray(rng.standard_normal(d1 + (2, nb)).astype(np.float32))
    uh = np.asfortranarray(rng.standard_normal(d1 + (3, 2, nb)).astype(np.float32))
    bnd = [(0, 1, 2), (2, 2, 1)]
    s, so = pkg.Settings(deg, bnd, 1), O.Sett.make(deg, bnd, 1)
    tf0, tphi, tug, tuh = (L.from_numpy(x) for x in (f0, phi, ug, uh))

    def run():
        out = (pkg.pull_hess(tf0, tphi, s), pkg.pull_grad_dot(tf0, tphi, tug, s), pkg.pull_hess_dot(tf0, tphi, tuh, s))
        torch.cuda.synchronize()
        return [L.to_numpy(x) for x in out]

    got_h, got_gd, got_hd = run()
    assert lib.pp_device_status(1) == 0
    assert got_h.shape == d1 + (3, 3, 2, nb) and got_gd.shape == phi.shape and got_hd.shape == phi.shape
    for b in range(nb):
        fb, pb = np.asfortranarray(f0[..., b]), np.asfortranarray(phi[..., b])
        h = O.pull_hess(fb, pb, so, threads=8)                    # (d1, 3, 3, C)
        g = O.pull_grad(fb, pb, so, threads=8)                    # (d1, 3, C)
        assert rel_err(got_h[..., b], h) <= 1e-4, (deg, b)
        ref_gd = np.einsum("xyzkc,xyzc->xyzk", g, ug[..., b].astype(np.float64))
        assert rel_err(got_gd[..., b], ref_gd) <= 1e-4, (deg, b)
        ref_hd = np.einsum("xyzpqc,xyzqc->xyzp", h, uh[..., b].astype(np.float64))
        assert rel_err(got_hd[..., b], ref_hd) <= 1e-4, (deg, b)
    assert lib.pp_set_path(1) == 0
    try:
        direct = run()
    finally:
        lib.pp_set_path(0)
    for got, ref in zip((got_h, got_gd, got_hd), direct):
        assert rel_err(got, ref) <= 1e-5
