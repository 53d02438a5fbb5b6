"""The host-pointer layer: the reference CPU library's own symbols (pull, pullg,
pullh, push, pushg with the signatures of artifacts/C/pushpull.h) called on host
numpy arrays exactly as src/pushpull_cpu.jl calls them, one (channel, batch)
slice at a time.  Checked against the reference's outputs (golden vectors) and,
on volumes large enough to be cut into pipelined slabs, against the native
device-pointer path; push accumulates into the caller's array."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = {"pull": 1e-5, "pullg": 1e-4, "pullh": 1e-4, "push": 1e-4, "pushg": 1e-4}
FL = C.POINTER(C.c_float)
U3 = C.c_ulonglong * 3


def _host_call(lib, sym, out, phi, inp, d0, n1, bnd, deg, ext):
    getattr(lib, sym)(out.ctypes.data_as(FL), phi.ctypes.data_as(FL), inp.ctypes.data_as(FL), U3(*d0),
                      C.c_ulonglong(n1), (C.c_int * 3)(*bnd), U3(*[d + 1 for d in deg]), C.c_int(ext))


def _slice(a, nd):
    """first (channel, batch) slice of a golden array: the first nd dims"""
    idx = (slice(None),) * nd + (0,) * (a.ndim - nd)
    return np.asfortranarray(a[idx])


def test_host_symbols_golden(pkg, golden):
    z, index = golden
    lib = pkg.native_library()
    for case in index["cases"]:
        nm = case["name"]
        deg, ext = tuple(case["deg"]), case["ext"]
        bnd = case["bnd"][0]
        f0 = _slice(z[f"{nm}/f0"], 3)
        phi = np.asfortranarray(z[f"{nm}/phi"])
        if phi.ndim > 4:
            phi = np.asfortranarray(phi[..., 0])
        f1 = _slice(z[f"{nm}/f1"], 3)
        g1 = _slice(z[f"{nm}/g1"], 4)
        d0, d1 = f0.shape[:3], phi.shape[:3]
        n1 = int(np.prod(d1))
        for op, sym, inp, shape in [("pull", "pull", f0, d1), ("pullg", "pullg", f0, d1 + (3,)),
                                    ("pullh", "pullh", f0, d1 + (3, 3)), ("push", "push", f1, d0),
                                    ("pushg", "pushg", g1, d0)]:
            key = f"{nm}/{op}"
            if key not in z.files:
                continue
            out = np.zeros(shape, dtype=np.float32, order="F")
            _host_call(lib, sym, out, phi, inp, d0, n1, bnd, deg, ext)
            ref = z[key]
            ref = ref.reshape(shape + ref.shape[len(shape):], order="F")
            ref = _slice(ref, len(shape)) if ref.ndim > len(shape) else ref
            assert rel_err(out, ref) <= TOL[op], (nm, op)


@pytest.mark.parametrize("d0,d1", [((192, 160, 128), (192, 160, 128)), ((96, 80, 64), (100, 90, 70))])
def test_host_symbols_pipelined_match_native(pkg, O, d0, d1):
    L = pkg.layout
    lib = pkg.native_library()
    rng = np.random.default_rng(3)
    f0 = np.asfortranarray(rng.random(d0, dtype=np.float32))
    phi = O.identity(d1).astype(np.float64)
    for k in range(3):
        phi[..., k] = 1 + (phi[..., k] - 1) * (d0[k] - 1) / max(d1[k] - 1, 1)
    phi = np.asfortranarray((phi + 2.0 * rng.standard_normal(phi.shape)).astype(np.float32))
    f1 = np.asfortranarray(rng.standard_normal(d1).astype(np.float32))
    n1 = int(np.prod(d1))
    s = pkg.Settings(3, 1, 1)
    out1 = np.zeros(d1, dtype=np.float32, order="F")
    _host_call(lib, "pull", out1, phi, f0, d0, n1, (1, 1, 1), (3, 3, 3), 1)
    ref1 = L.to_numpy(pkg.pull(L.from_numpy(f0), L.from_numpy(phi), s))
    # the same kernels when the grid is inferred exactly; otherwise the per-voxel
    # kernels, whose summation order differs from the tiled ones
    exact = tuple(d0) == tuple(d1)
    assert np.array_equal(out1, ref1) if exact else rel_err(out1, ref1) <= 1e-6
    acc = np.full(d0, 0.5, dtype=np.float32, order="F")            # push adds into the caller's array
    _host_call(lib, "push", acc, phi, f1, d0, n1, (1, 1, 1), (3, 3, 3), 1)
    ref0 = L.to_numpy(pkg.push(L.from_numpy(f1), L.from_numpy(phi), d0, s)) + np.float32(0.5)
    assert rel_err(acc, ref0) <= 1e-5
    g = np.asfortranarray(rng.standard_normal(d1 + (3,)).astype(np.float32))
    outg = np.zeros(d1 + (3,), dtype=np.float32, order="F")
    _host_call(lib, "pullg", outg, phi, f0, d0, n1, (1, 1, 1), (3, 3, 3), 1)
    refg = L.to_numpy(pkg.pull_grad(L.from_numpy(f0), L.from_numpy(phi), s))
    assert np.array_equal(outg, refg) if exact else rel_err(outg, refg) <= 1e-6
    accg = np.zeros(d0, dtype=np.float32, order="F")
    _host_call(lib, "pushg", accg, phi, g, d0, n1, (1, 1, 1), (3, 3, 3), 1)
    assert rel_err(accg, L.to_numpy(pkg.push_grad(L.from_numpy(g), L.from_numpy(phi), d0, s))) <= 1e-5
