"""Affine pull / push (pp_pull_affine, pp_push_affine and the reference-named
host symbols pull_affine / push_affine) against the reference's own outputs
(golden vectors), the FP64 oracle and the adjoint identity.

Tolerances as for the deformation ops: pull 1e-5, push 1e-4 (norm-wise
relative, NaN masks identical); degree-0 pull bit-exact against the reference;
adjoint |<pull(a), b> - <a, push(b)>| <= 1e-5 relative (sums in float64)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest
import torch

from conftest import golden_sett, rel_err

pytestmark = pytest.mark.gpu


def _sett(pkg, case):
    bnd = [tuple(b) for b in case["bnd"]]
    return pkg.Settings(tuple(case["deg"]), bnd if len(bnd) > 1 else bnd[0], case["ext"])


def test_affine_golden(pkg, O, golden):
    z, index = golden
    L = pkg.layout
    for case in index["affine"]:
        nm = case["name"]
        s, so = _sett(pkg, case), golden_sett(O, case)
        A, f0, f1 = z[f"{nm}/A"], z[f"{nm}/f0"], z[f"{nm}/f1"]
        got1 = L.to_numpy(pkg.affine_pull(L.from_numpy(f0), A, case["d1"], s))
        got0 = L.to_numpy(pkg.affine_push(L.from_numpy(f1), A, case["d0"], s))
        ref1, ref0 = z[f"{nm}/pull_affine"], z[f"{nm}/push_affine"]
        if tuple(case["deg"]) == (0, 0, 0):
            assert np.array_equal(got1, ref1, equal_nan=True), nm
        assert rel_err(got1, ref1) <= 1e-5, nm
        assert rel_err(got0, ref0) <= 1e-4, nm
        assert rel_err(got1, O.pull_affine(f0, A, case["d1"], so)) <= 1e-5, nm
        assert rel_err(got0, O.push_affine(f1, A, case["d0"], so)) <= 1e-4, nm


def _affine(rng, d0, d1):
    """1-based 4x4 map from the d1 grid into the d0 grid: rotation, scaling, shift."""
    th = rng.uniform(-0.3, 0.3, 3)
    cx, sx = np.cos(th), np.sin(th)
    R = (np.array([[1, 0, 0], [0, cx[0], -sx[0]], [0, sx[0], cx[0]]])
         @ np.array([[cx[1], 0, sx[1]], [0, 1, 0], [-sx[1], 0, cx[1]]])
         @ np.array([[cx[2], -sx[2], 0], [sx[2], cx[2], 0], [0, 0, 1]]))
    S = np.diag([(d0[k] - 1) / max(d1[k] - 1, 1) for k in range(3)])
    M = R @ S
    c0 = 0.5 * (np.array(d0) + 1)
    c1 = 0.5 * (np.array(d1) + 1)
    t = c0 - M @ c1 + rng.uniform(-2, 2, 3)
    A = np.eye(4, dtype=np.float32)
    A[:3, :3] = M
    A[:3, 3] = t
    return A


@pytest.mark.parametrize("deg,bnd,ext", [(0, 1, 0), (1, 0, 0), (2, (0, 1, 2), 1), (3, 1, 1), (4, 2, 1),
                                         ((1, 3, 2), 1, 1)])
def test_affine_vs_oracle_multichannel(pkg, O, deg, bnd, ext):
    L = pkg.layout
    rng = np.random.default_rng(31)
    d0, d1 = (29, 23, 19), (17, 21, 13)
    A = _affine(rng, d0, d1)
    f0 = np.asfortranarray(rng.standard_normal(d0 + (2, 2)).astype(np.float32))
    f1 = np.asfortranarray(rng.standard_normal(d1 + (2, 2)).astype(np.float32))
    s, so = pkg.Settings(deg, bnd, ext), O.Sett.make(deg, bnd, ext)
    got1 = L.to_numpy(pkg.affine_pull(L.from_numpy(f0), A, d1, s))
    got0 = L.to_numpy(pkg.affine_push(L.from_numpy(f1), A, d0, s))
    assert rel_err(got1, O.pull_affine(f0, A, d1, so)) <= 1e-5
    assert rel_err(got0, O.push_affine(f1, A, d0, so)) <= 1e-4


def test_affine_adjoint_and_accumulate(pkg):
    L = pkg.layout
    rng = np.random.default_rng(32)
    d0, d1 = (64, 48, 40), (57, 61, 33)
    A = _affine(rng, d0, d1)
    s = pkg.Settings(3, 1, 1)
    a = L.empty(d0, device="cuda").normal_()
    b = L.empty(d1, device="cuda").normal_()
    lhs = float((pkg.affine_pull(a, A, d1, s).double() * b.double()).sum())
    pb = pkg.affine_push(b, A, d0, s)
    rhs = float((a.double() * pb.double()).sum())
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)
    acc = pb.clone()
    pkg.affine_push(b, A, d0, s, out=acc, accumulate=True)
    assert torch.allclose(acc, 2 * pb, rtol=1e-5, atol=1e-5 * float(pb.abs().max()))


def test_affine_host_symbols(pkg, O, golden):
    """pull_affine / push_affine with the reference CPU signature on host arrays."""
    z, index = golden
    lib = pkg.native_library()
    fl = C.POINTER(C.c_float)
    u64 = C.c_ulonglong * 3
    for case in index["affine"]:
        nm = case["name"]
        if len(case["bnd"]) > 1:
            continue
        A = O.adjust_affine(z[f"{nm}/A"])
        Af = np.asfortranarray(A).reshape(-1, order="F").astype(np.float32)
        f0 = np.asfortranarray(z[f"{nm}/f0"][..., 0] if z[f"{nm}/f0"].ndim > 3 else z[f"{nm}/f0"])
        f1 = np.asfortranarray(z[f"{nm}/f1"][..., 0] if z[f"{nm}/f1"].ndim > 3 else z[f"{nm}/f1"])
        d0, d1 = tuple(case["d0"]), tuple(case["d1"])
        bnd = (C.c_int * 3)(*case["bnd"][0])
        dp = u64(*[d + 1 for d in case["deg"]])
        out1 = np.zeros(d1, dtype=np.float32, order="F")
        lib.pull_affine(out1.ctypes.data_as(fl), f0.ctypes.data_as(fl), u64(*d0), C.c_ulonglong(int(np.prod(d1))),
                        u64(*d1), Af.ctypes.data_as(fl), bnd, dp, C.c_int(case["ext"]))
        out0 = np.zeros(d0, dtype=np.float32, order="F")
        lib.push_affine(out0.ctypes.data_as(fl), f1.ctypes.data_as(fl), u64(*d0), C.c_ulonglong(int(np.prod(d1))),
                        u64(*d1), Af.ctypes.data_as(fl), bnd, dp, C.c_int(case["ext"]))
        so = golden_sett(O, case)
        assert rel_err(out1, O.pull_affine(f0, z[f"{nm}/A"], d1, so)) <= 1e-5, nm
        assert rel_err(out0, O.push_affine(f1, z[f"{nm}/A"], d0, so)) <= 1e-4, nm
