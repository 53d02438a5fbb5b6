"""Both kernel families (shared-memory tiled, per-voxel global) against the FP64
oracle on moderate volumes, across tile shapes, forced per-tile fallbacks (tiny
shared-memory budgets), multiple channels with per-channel boundaries, and
batches.  Tolerances as in test_gpu_parity: pull 1e-5, the rest 1e-4."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = {"pull": 1e-5, "pullg": 1e-4, "pullh": 1e-4, "push": 1e-4, "pushg": 1e-4}


def _phi(O, rng, d1, d0, sigma, nb=1):
    out = []
    for _ in range(nb):
        p = O.identity(d1).astype(np.float64)
        for k in range(3):
            p[..., k] = 1 + (p[..., k] - 1) * (d0[k] - 1) / max(d1[k] - 1, 1)
        out.append(p + sigma * rng.standard_normal(p.shape))
    a = np.stack(out, axis=-1) if nb > 1 else out[0]
    return np.asfortranarray(a.astype(np.float32))


@pytest.fixture
def restore_tiles(pkg):
    lib = pkg.native_library()
    saved = {}
    for op in range(6):
        for d in range(5):
            v = [C.c_int() for _ in range(4)]
            assert lib.pp_get_tile(op, d, *[C.byref(x) for x in v]) == 0
            saved[(op, d)] = [x.value for x in v]
    yield lib
    for (op, d), v in saved.items():
        lib.pp_set_tile(op, d, *v)
    lib.pp_set_path(0)


def _all_ops(pkg, O, f0, phi, f1, g1, s_pkg, s_ora):
    L = pkg.layout
    d0 = f0.shape[:3]
    tf0, tphi, tf1, tg1 = (L.from_numpy(a) for a in (f0, phi, f1, g1))
    got = {
        "pull": pkg.pull(tf0, tphi, s_pkg), "pullg": pkg.pull_grad(tf0, tphi, s_pkg),
        "pullh": pkg.pull_hess(tf0, tphi, s_pkg), "push": pkg.push(tf1, tphi, d0, s_pkg),
        "pushg": pkg.push_grad(tg1, tphi, d0, s_pkg),
    }
    torch.cuda.synchronize()
    ref = {
        "pull": O.pull(f0, phi, s_ora), "pullg": O.pull_grad(f0, phi, s_ora),
        "pullh": O.pull_hess(f0, phi, s_ora), "push": O.push(f1, phi, d0, s_ora),
        "pushg": O.push_grad(g1, phi, d0, s_ora),
    }
    for k in got:
        e = rel_err(L.to_numpy(got[k]), ref[k])
        assert e <= TOL[k], (k, e)


@pytest.mark.parametrize("tile", [(3, 3, 3, 12288), (5, 2, 2, 12288), (4, 3, 1, 8192), (2, 2, 2, 4096),
                                  (3, 3, 3, 64)])
@pytest.mark.parametrize("deg,bnd,ext", [(1, 0, 0), (3, 1, 1), (2, (0, 1, 2), 1), (4, 2, 1), (0, 1, 0)])
def test_tiled_vs_oracle(pkg, O, restore_tiles, tile, deg, bnd, ext):
    lib = restore_tiles
    assert lib.pp_set_tile(-1, -1, *tile) == 0
    rng = np.random.default_rng(deg * 7 + tile[0])
    d0, d1 = (37, 29, 23), (33, 27, 19)
    f0 = np.asfortranarray(rng.standard_normal(d0 + (2,)).astype(np.float32))
    phi = _phi(O, rng, d1, d0, 2.0)
    f1 = np.asfortranarray(rng.standard_normal(d1 + (2,)).astype(np.float32))
    g1 = np.asfortranarray(rng.standard_normal(d1 + (3, 2)).astype(np.float32))
    _all_ops(pkg, O, f0, phi, f1, g1, pkg.Settings(deg, bnd, ext), O.Sett.make(deg, bnd, ext))


@pytest.mark.parametrize("path", [0, 1])
def test_paths_multichannel_batch(pkg, O, restore_tiles, path):
    """Per-channel boundaries, 3 channels, batch 2, anisotropic and isotropic degrees."""
    lib = restore_tiles
    assert lib.pp_set_path(path) == 0
    rng = np.random.default_rng(11 + path)
    d0, d1, nb = (30, 26, 21), (28, 24, 17), 2
    f0 = np.asfortranarray(rng.standard_normal(d0 + (3, nb)).astype(np.float32))
    phi = _phi(O, rng, d1, d0, 1.5, nb=nb)
    f1 = np.asfortranarray(rng.standard_normal(d1 + (3, nb)).astype(np.float32))
    g1 = np.asfortranarray(rng.standard_normal(d1 + (3, 3, nb)).astype(np.float32))
    bnd = [(0, 0, 0), (1, 2, 1), (2, 1, 0)]
    for deg in [(3, 3, 3), (1, 3, 2)]:
        _all_ops(pkg, O, f0, phi, f1, g1, pkg.Settings(deg, bnd, 1), O.Sett.make(deg, bnd, 1))


def test_nonfinite_and_far_coordinates(pkg, O):
    """NaN/Inf deformations, far-out coordinates (fallback tiles) and NaN values."""
    rng = np.random.default_rng(5)
    d0, d1 = (24, 20, 16), (24, 20, 16)
    f0 = np.asfortranarray(rng.standard_normal(d0).astype(np.float32))
    phi = _phi(O, rng, d1, d0, 1.0)
    phi[3, 4, 5, 0] = np.nan
    phi[10, 2, 7, 1] = np.inf
    phi[20:24, 0:8, 0:8, 2] += 1e4                    # one tile far away: its box cannot fit
    f1 = np.asfortranarray(rng.standard_normal(d1).astype(np.float32))
    f1[5, 5, 5] = np.nan
    g1 = np.asfortranarray(rng.standard_normal(d1 + (3,)).astype(np.float32))
    for deg, bnd, ext in [(3, 1, 1), (2, 0, 1), (1, 2, 0)]:
        _all_ops(pkg, O, f0, phi, f1, g1, pkg.Settings(deg, bnd, ext), O.Sett.make(deg, bnd, ext))


def test_identity_reproduces_image(pkg, O):
    """pull at the identity grid returns the image itself for degrees 0 and 1."""
    L = pkg.layout
    rng = np.random.default_rng(9)
    d = (19, 17, 13)
    f0 = np.asfortranarray(rng.standard_normal(d).astype(np.float32))
    phi = L.from_numpy(O.identity(d))
    for deg in (0, 1):
        out = L.to_numpy(pkg.pull(L.from_numpy(f0), phi, pkg.Settings(deg, 1, 0)))
        assert np.array_equal(out, f0)


def test_autotune_installs_valid_choice(pkg, O, restore_tiles, tmp_path, monkeypatch):
    """The autotuner times candidates on the caller's arrays, installs a tile
    configuration that still matches the oracle, and caches it."""
    import importlib
    A = importlib.import_module("pushpull_gb300.autotune")
    monkeypatch.setattr(A, "CACHE", str(tmp_path / "tiles.json"))
    L = pkg.layout
    rng = np.random.default_rng(21)
    d0 = d1 = (48, 40, 36)
    f0 = np.asfortranarray(rng.standard_normal(d0).astype(np.float32))
    phi = _phi(O, rng, d1, d0, 1.5)
    s, so = pkg.Settings(3, 1, 1), O.Sett.make(3, 1, 1)
    for op, x in [("pull", f0), ("push", f0)]:
        res = A.tune(op, L.from_numpy(x), L.from_numpy(phi), s, d0=d0, reps=2)
        assert res["path"] in ("tiled", "direct") and res["ms"] > 0
        assert sum(res["tile"]) >= 6
        assert res["cap"] >= 4096 if res["path"] == "tiled" else res["cap"] == 0
    got1 = L.to_numpy(pkg.pull(L.from_numpy(f0), L.from_numpy(phi), s))
    got0 = L.to_numpy(pkg.push(L.from_numpy(f0), L.from_numpy(phi), d0, s))
    assert rel_err(got1, O.pull(f0, phi, so)) <= 1e-5
    assert rel_err(got0, O.push(f0, phi, d0, so)) <= 1e-4
    assert A.load() == len(__import__("json").load(open(A.CACHE)))
