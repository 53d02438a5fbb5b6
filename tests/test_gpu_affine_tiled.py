"""Affine pull / push on the tiled kernels (positions A (i, j, k, 1) computed in
the warp-specialised pull and in the tiled push, no deformation read) against
the FP64 oracle and against the per-voxel affine kernels, on every path a tile
can take:

* near-identity maps (interior TMA windows, mirrored and circulant margins);
* strong contraction (many voxels per box element: the warp-cooperative scatter
  of the push) and strong expansion (boxes larger than a buffer: per-voxel
  fallback inside the tiled kernels);
* ext = 0 with positions leaving the band (NaN outputs, skipped pushes),
  several channels with per-channel bounds, batches, degrees 1..4 (degree 1
  forced onto the tiled kernels with pp_set_tile);
* the full 192^3 cubic benchmark map.
Tolerances as for the deformation ops: pull 1e-5, push 1e-4 (norm-wise
relative), NaN masks identical."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture
def tiles(pkg):
    lib = pkg.native_library()
    saved = {}
    for op in range(6):
        for d in range(5):
            v = [C.c_int() for _ in range(4)]
            assert lib.pp_get_tile(op, d, *[C.byref(x) for x in v]) == 0
            saved[(op, d)] = [x.value for x in v]
    # degree 1 onto the tiled kernels as well (pull: the warp-specialised code)
    assert lib.pp_set_tile(0, 1, 3, 3, 4, 15360) == 0, lib.pp_last_error()
    assert lib.pp_set_tile(3, 1, 3, 3, 3, 16384) == 0, lib.pp_last_error()
    yield lib
    for (op, d), v in saved.items():
        lib.pp_set_tile(op, d, *v)
    lib.pp_set_path(0)


def _map(rng, d0, d1, zoom=1.0, rot=0.3, shift=2.0):
    """1-based 4x4 map of the d1 grid into the d0 grid (rotation, zoom about the centres, shift)."""
    th = rng.uniform(-rot, rot, 3)
    c, s = np.cos(th), np.sin(th)
    R = (np.array([[1, 0, 0], [0, c[0], -s[0]], [0, s[0], c[0]]])
         @ np.array([[c[1], 0, s[1]], [0, 1, 0], [-s[1], 0, c[1]]])
         @ np.array([[c[2], -s[2], 0], [s[2], c[2], 0], [0, 0, 1]]))
    M = R @ np.diag([zoom * (d0[k] - 1) / max(d1[k] - 1, 1) for k in range(3)])
    c0, c1 = 0.5 * (np.array(d0) + 1), 0.5 * (np.array(d1) + 1)
    A = np.eye(4, dtype=np.float32)
    A[:3, :3] = M
    A[:3, 3] = c0 - M @ c1 + rng.uniform(-shift, shift, 3)
    return A


def _both(pkg, lib, f0, f1, A, d0, d1, s):
    """(pull, push) on the default (tiled) path and on the per-voxel kernels."""
    L = pkg.layout
    t0, t1 = L.from_numpy(f0), L.from_numpy(f1)
    got = (L.to_numpy(pkg.affine_pull(t0, A, d1, s)), L.to_numpy(pkg.affine_push(t1, A, d0, s)))
    assert lib.pp_set_path(1) == 0
    try:
        ref = (L.to_numpy(pkg.affine_pull(t0, A, d1, s)), L.to_numpy(pkg.affine_push(t1, A, d0, s)))
    finally:
        lib.pp_set_path(0)
    assert lib.pp_device_status(1) == 0
    return got, ref


@pytest.mark.parametrize("deg,bnd,ext,zoom", [(1, 0, 1, 1.0), (2, (0, 1, 2), 1, 1.0), (3, 1, 1, 1.0), (4, 2, 1, 1.0),
                                              (3, 1, 0, 1.3), (3, 1, 1, 0.15), (2, 0, 1, 6.0), (4, 1, 1, 0.3)])
def test_affine_tiled_vs_oracle(pkg, O, tiles, deg, bnd, ext, zoom):
    rng = np.random.default_rng(100 + deg)
    d0, d1 = (44, 40, 36), (48, 36, 40)
    A = _map(rng, d0, d1, zoom=zoom)
    f0 = np.asfortranarray(rng.standard_normal(d0 + (2, 2)).astype(np.float32))
    f1 = np.asfortranarray(rng.standard_normal(d1 + (2, 2)).astype(np.float32))
    s, so = pkg.Settings(deg, bnd, ext), O.Sett.make(deg, bnd, ext)
    (g1, g0), (r1, r0) = _both(pkg, tiles, f0, f1, A, d0, d1, s)
    o1, o0 = O.pull_affine(f0, A, d1, so), O.push_affine(f1, A, d0, so)
    assert np.array_equal(np.isnan(g1), np.isnan(o1))
    assert rel_err(g1, o1) <= 1e-5
    assert rel_err(g0, o0) <= 1e-4
    # the per-voxel kernels: same positions, other summation order
    assert np.array_equal(np.isnan(g1), np.isnan(r1))
    assert rel_err(g1, r1) <= 1e-5
    assert rel_err(g0, r0) <= 1e-4


def test_affine_tiled_degree0_bit_exact(pkg, O, tiles):
    """Nearest neighbour through the tiled paths is bit-exact against the reference rounding."""
    lib = tiles
    assert lib.pp_set_tile(0, 0, 3, 3, 4, 15360) == 0 and lib.pp_set_tile(3, 0, 3, 3, 3, 16384) == 0
    rng = np.random.default_rng(7)
    d0, d1 = (40, 36, 32), (40, 36, 32)
    A = _map(rng, d0, d1, zoom=1.1)
    f0 = np.asfortranarray(rng.standard_normal(d0).astype(np.float32))
    f1 = np.asfortranarray(rng.standard_normal(d1).astype(np.float32))
    s, so = pkg.Settings(0, 1, 0), O.Sett.make(0, 1, 0)
    (g1, g0), _ = _both(pkg, lib, f0, f1, A, d0, d1, s)
    assert np.array_equal(g1, O.pull_affine(f0, A, d1, so, kind="ref").astype(np.float32), equal_nan=True)
    assert rel_err(g0, O.push_affine(f1, A, d0, so)) <= 1e-4


def test_affine_192_cubic_vs_oracle_and_adjoint(pkg, O):
    """The benchmarked map at full size: FP64 oracle and <pull(a), b> = <a, push(b)>."""
    from pushpull_gb300 import workloads as W
    L = pkg.layout
    w = W.config2()
    d = tuple(w.f0.shape[:3])
    A = W.affine_map(d, seed=6)
    s, so = pkg.Settings(3, 1, 1), O.Sett.make(3, 1, 1)
    f1 = L.to_numpy(pkg.affine_pull(L.from_numpy(w.f0), A, d, s))
    assert rel_err(f1, O.pull_affine(w.f0, A, d, so)) <= 1e-5
    f0b = L.to_numpy(pkg.affine_push(L.from_numpy(f1), A, d, s))
    assert rel_err(f0b, O.push_affine(f1, A, d, so)) <= 1e-4
    lhs = float(np.sum(f1.astype(np.float64) * f1))
    rhs = float(np.sum(w.f0.astype(np.float64) * f0b))
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)
