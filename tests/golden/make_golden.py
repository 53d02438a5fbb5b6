"""Generate the golden vectors in ``pushpull_golden.npz`` from the reference itself.

Run where the reference tree is present:  ``python tests/golden/make_golden.py``.
It compiles the reference's CPU library from its C sources (``oracle/build.py``)
and records its outputs on seeded Float32 inputs:

* ``pull``, ``pullg``, ``pullh``, ``push`` straight from the reference symbols;
* ``pushg`` (push_grad) as the exact transpose of the reference ``pullg``: the
  reference CPU ``pushg`` adds nothing for finite input (artifacts/C/pushpull.c:144),
  so its golden values are built column by column from ``pullg`` applied to unit
  volumes and contracted with the input gradient field in float64;
* ``pull_affine`` / ``push_affine`` from the reference affine symbols.

Cases cover every degree, boundary and extrapolate setting, anisotropic degrees,
per-channel boundaries, size-1 dimensions, degree-0 ties at half-integers, the
ext = 0 band edges, non-finite deformations and values, far-out coordinates, and
the reference test suite's own setting (test/runtests.jl:44-95).
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402

OUT = os.path.join(HERE, "pushpull_golden.npz")


def f32(a):
    return np.asfortranarray(np.asarray(a, dtype=np.float32))


def rand_phi(rng, d1, d0, sigma, nb=None):
    phi = O.identity(d1).astype(np.float64)
    # stretch the identity so the deformed grid spans the source volume
    for k in range(3):
        phi[..., k] = 1.0 + (phi[..., k] - 1.0) * (d0[k] - 1) / max(d1[k] - 1, 1)
    if nb is None:
        return f32(phi + sigma * rng.standard_normal(phi.shape))
    return f32(np.stack([phi + sigma * rng.standard_normal(phi.shape) for _ in range(nb)], axis=-1))


def pushg_from_pullg(g1, phi, d0, sett):
    """push_grad as the transpose of the reference pull_grad (one batch, C channels)."""
    nc = g1.shape[4] if g1.ndim > 4 else 1
    g1_shape = g1.shape
    g1 = g1.reshape(g1.shape[:4] + (nc,), order="F")
    n0 = int(np.prod(d0))
    d1 = phi.shape[:3]
    out = np.zeros(tuple(d0) + (nc,), dtype=np.float64, order="F")
    for c in range(nc):
        sc = O.Sett.make(sett.deg, sett.bnd_for(c), sett.ext)
        cols = []
        for j in range(n0):
            e = np.zeros(n0, dtype=np.float32)
            e[j] = 1.0
            cols.append(O.pull_grad(f32(e.reshape(d0, order="F")), phi, sc, "ref").reshape(-1, order="F"))
        M = np.stack(cols, axis=1).astype(np.float64)        # (3 n1, n0)
        g = g1[..., c].reshape(-1, order="F").astype(np.float64)
        n1 = int(np.prod(d1))
        ok = np.isfinite(M).all(axis=1).reshape(3, n1).all(axis=0)   # valid voxels
        ok &= np.isfinite(g).reshape(3, n1).all(axis=0)              # finite gradients
        keep = np.tile(ok, 3)
        out[..., c] = (M[keep].T @ g[keep]).reshape(d0, order="F")
    return np.asfortranarray(out.reshape(tuple(d0) + tuple(g1_shape[4:]), order="F").astype(np.float32))


def main():
    if not O.ref_available():
        raise SystemExit("reference sources not present: cannot generate golden vectors")
    rng = np.random.default_rng(20240607)
    cases = []
    arrays = {}

    def add(name, deg, bnd, ext, f0, phi, f1, g1, ops=("pull", "pullg", "pullh", "push", "pushg")):
        s = O.Sett.make(deg, bnd, ext)
        d0 = f0.shape[:3]
        arrays[f"{name}/f0"] = f0
        arrays[f"{name}/phi"] = phi
        arrays[f"{name}/f1"] = f1
        arrays[f"{name}/g1"] = g1
        if "pull" in ops:
            arrays[f"{name}/pull"] = O.pull(f0, phi, s, "ref")
        if "pullg" in ops:
            arrays[f"{name}/pullg"] = O.pull_grad(f0, phi, s, "ref")
        if "pullh" in ops:
            arrays[f"{name}/pullh"] = O.pull_hess(f0, phi, s, "ref")
        if "push" in ops:
            arrays[f"{name}/push"] = O.push(f1, phi, d0, s, "ref")
        if "pushg" in ops:
            nb = phi.shape[4] if phi.ndim == 5 else 1
            if nb == 1:
                arrays[f"{name}/pushg"] = pushg_from_pullg(g1, phi[..., :3] if phi.ndim == 4 else phi[..., 0], d0, s)
        cases.append(dict(name=name, deg=list(s.deg), bnd=[list(b) for b in s.bnd], ext=s.ext,
                          ops=[o for o in ops if f"{name}/{o}" in arrays]))

    # 1. every isotropic degree x boundary x extrapolate on a small non-cubic pair
    d0, d1 = (7, 6, 5), (5, 6, 4)
    for deg in range(5):
        for bnd in (0, 1, 2, (0, 1, 2)):
            for ext in (0, 1):
                f0 = f32(rng.standard_normal(d0))
                phi = rand_phi(rng, d1, d0, 1.2)
                phi[0, 0, 0, 0] = np.nan                  # non-finite deformation
                phi[1, 0, 0, 1] = np.inf
                phi[2, 1, 0, 2] = -60.3                   # far outside (ext=1 wraps)
                phi[3, 2, 1, 0] = 45.7
                f1 = f32(rng.standard_normal(d1))
                f1[4, 5, 3] = np.nan                      # non-finite value: push skips
                g1 = f32(rng.standard_normal(d1 + (3,)))
                g1[0, 1, 2, 1] = np.inf                   # non-finite gradient: push_grad skips
                b = bnd if isinstance(bnd, tuple) else (bnd,) * 3
                add(f"iso_d{deg}_b{''.join(map(str, b))}_e{ext}", deg, bnd, ext, f0, phi, f1, g1)

    # 2. anisotropic degrees with mixed boundaries
    for deg, bnd in (((0, 2, 4), (2, 0, 1)), ((1, 3, 2), (1, 2, 0)), ((4, 0, 3), (0, 2, 2)),
                     ((3, 1, 0), (2, 1, 0))):
        for ext in (0, 1):
            f0 = f32(rng.standard_normal(d0))
            phi = rand_phi(rng, d1, d0, 1.5)
            f1 = f32(rng.standard_normal(d1))
            g1 = f32(rng.standard_normal(d1 + (3,)))
            add(f"aniso_d{''.join(map(str, deg))}_b{''.join(map(str, bnd))}_e{ext}", deg, bnd, ext,
                f0, phi, f1, g1)

    # 3. per-channel boundaries, 3 channels
    for deg in (1, 3):
        f0 = f32(rng.standard_normal(d0 + (3,)))
        phi = rand_phi(rng, d1, d0, 2.0)
        f1 = f32(rng.standard_normal(d1 + (3,)))
        g1 = f32(rng.standard_normal(d1 + (3, 3)))
        add(f"perchan_d{deg}", deg, [(0, 0, 0), (1, 1, 1), (2, 1, 0)], 1, f0, phi, f1, g1)

    # 4. size-1 dimensions (the reference tests use d3 = 1)
    for dd0, dd1 in (((8, 7, 1), (8, 7, 1)), ((1, 5, 1), (3, 4, 2)), ((4, 1, 3), (2, 2, 2)),
                     ((1, 1, 1), (2, 3, 1))):
        for deg in (0, 2, 3):
            f0 = f32(rng.standard_normal(dd0))
            phi = rand_phi(rng, dd1, dd0, 1.0)
            f1 = f32(rng.standard_normal(dd1))
            g1 = f32(rng.standard_normal(dd1 + (3,)))
            add(f"size1_{'x'.join(map(str, dd0))}_d{deg}", deg, (0, 1, 2), 1, f0, phi, f1, g1)

    # 5. the reference test suite's setting: d=(8,7,1), c=2, deg 2/3, bnd (0,1,2), ext=1, batch 2
    d = (8, 7, 1)
    for deg in (2, 3):
        f0 = f32(rng.standard_normal(d + (2, 2)))
        phi = f32(np.stack([O.identity(d) + rng.standard_normal(d + (3,)).astype(np.float32)
                            for _ in range(2)], axis=-1))
        f1 = f32(rng.standard_normal(d + (2, 2)))
        g1 = f32(rng.standard_normal(d + (3, 2, 2)))
        add(f"reftest_d{deg}_batch2", deg, (0, 1, 2), 1, f0, phi, f1, g1,
            ops=("pull", "pullg", "pullh", "push"))

    # 6. degree-0 and degree-1 ties at half-integers / integers, and ext=0 band edges
    d0t, d1t = (6, 5, 4), (8, 1, 1)
    f0 = f32(rng.standard_normal(d0t))
    base = np.array([1.5, 2.5, 3.5, 0.99, 1.0, 2.0, 5.01, 5.0], dtype=np.float32)
    nxt = np.nextafter(base, np.float32(10)).astype(np.float32)
    prv = np.nextafter(base, np.float32(-10)).astype(np.float32)
    for tag, xs in (("exact", base), ("up", nxt), ("down", prv)):
        phi = np.zeros(d1t + (3,), dtype=np.float32, order="F")
        phi[:, 0, 0, 0] = xs
        phi[:, 0, 0, 1] = np.array([1.0, 1.5, 2.5, 0.99, 5.01, 4.99, 1.0, 5.0], np.float32)[: d1t[0]]
        phi[:, 0, 0, 2] = np.array([0.99, 4.01, 3.99, 1.0, 2.5, 3.5, 4.0, 1.0], np.float32)[: d1t[0]]
        phi = f32(phi)
        f1 = f32(rng.standard_normal(d1t))
        g1 = f32(rng.standard_normal(d1t + (3,)))
        for deg in (0, 1):
            for ext in (0, 1):
                add(f"ties_{tag}_d{deg}_e{ext}", deg, 1, ext, f0, phi, f1, g1)

    # 7. far-out coordinates with extrapolation (wrap / mirror many periods away)
    f0 = f32(rng.standard_normal(d0))
    phi = f32(rand_phi(rng, d1, d0, 1.0) + rng.choice([-97.0, -31.0, 23.0, 71.0], size=d1 + (3,)))
    f1 = f32(rng.standard_normal(d1))
    g1 = f32(rng.standard_normal(d1 + (3,)))
    for deg in (1, 3, 4):
        for bnd in (0, 1, 2):
            add(f"far_d{deg}_b{bnd}", deg, bnd, 1, f0, phi, f1, g1)

    # 8. affine pull / push (artifacts/C/pushpull.c:176-244)
    aff_cases = []
    for deg, bnd, ext in ((1, 1, 1), (3, 0, 1), (2, 2, 0), (0, 1, 0)):
        A = np.array([[0.9, 0.1, -0.05, 0.7], [-0.08, 1.1, 0.03, -0.4], [0.02, -0.06, 0.95, 0.3]],
                     dtype=np.float32)
        s = O.Sett.make(deg, bnd, ext)
        f0 = f32(rng.standard_normal(d0 + (2,)))
        f1 = f32(rng.standard_normal(d1 + (2,)))
        name = f"affine_d{deg}_b{bnd}_e{ext}"
        arrays[f"{name}/A"] = A
        arrays[f"{name}/f0"] = f0
        arrays[f"{name}/f1"] = f1
        arrays[f"{name}/pull_affine"] = O.pull_affine(f0, A, d1, s, "ref")
        arrays[f"{name}/push_affine"] = O.push_affine(f1, A, d0, s, "ref")
        aff_cases.append(dict(name=name, deg=list(s.deg), bnd=[list(b) for b in s.bnd], ext=s.ext,
                              d0=list(d0), d1=list(d1)))

    index = dict(cases=cases, affine=aff_cases,
                 source="reference artifacts/C/pushpull.c compiled with gcc -O3 -ffp-contract=off")
    arrays["__index__"] = np.frombuffer(json.dumps(index).encode(), dtype=np.uint8)
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {OUT}: {len(cases)} cases + {len(aff_cases)} affine, "
          f"{os.path.getsize(OUT) / 1024:.0f} KiB")


if __name__ == "__main__":
    main()
