"""Pin the CPU oracle to the reference: golden vectors made by the reference's own
C library (tests/golden/make_golden.py).  Tolerances: the FP64 oracle within
1e-5 (norm-wise relative) of every reference output, NaN masks identical, and
degree-0 pulls bit-exact.  The FP32 port within 1e-5 as well."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_sett, rel_err

TOL = 1e-5


def _cases(golden):
    return golden[1]["cases"]


def test_golden_index_complete(golden):
    z, index = golden
    names = {c["name"] for c in index["cases"]}
    degs = {tuple(c["deg"]) for c in index["cases"]}
    assert {(d, d, d) for d in range(5)} <= degs
    assert any(c["ext"] == 0 for c in index["cases"]) and any(c["ext"] == 1 for c in index["cases"])
    assert any(len(c["bnd"]) > 1 for c in index["cases"])              # per-channel boundaries
    assert any(n.startswith("size1_") for n in names)
    assert any(n.startswith("ties_") for n in names)
    assert len(index["affine"]) >= 4


@pytest.mark.parametrize("op", ["pull", "pullg", "pullh", "push", "pushg"])
def test_oracle_matches_reference(golden, O, op):
    z, index = golden
    worst, n = 0.0, 0
    for case in index["cases"]:
        key = f"{case['name']}/{op}"
        if key not in z.files:
            continue
        s = golden_sett(O, case)
        f0, phi, f1, g1 = (z[f"{case['name']}/{k}"] for k in ("f0", "phi", "f1", "g1"))
        d0 = f0.shape[:3]
        if op == "pull":
            got = O.pull(f0, phi, s)
        elif op == "pullg":
            got = O.pull_grad(f0, phi, s)
        elif op == "pullh":
            got = O.pull_hess(f0, phi, s)
        elif op == "push":
            got = O.push(f1, phi, d0, s)
        else:
            got = O.push_grad(g1, phi, d0, s)
        ref = z[key]
        e = rel_err(got, ref)
        assert e <= TOL, (case["name"], op, e)
        if op == "pull" and case["deg"] == [0, 0, 0]:
            m = ~np.isnan(ref)
            assert np.array_equal(got[m].astype(np.float32), ref[m]), case["name"]
        worst, n = max(worst, e), n + 1
    assert n > 0


def test_port_matches_reference(golden, O):
    z, index = golden
    for case in index["cases"]:
        s = golden_sett(O, case)
        nm = case["name"]
        f0, phi, f1, g1 = (z[f"{nm}/{k}"] for k in ("f0", "phi", "f1", "g1"))
        assert rel_err(O.pull(f0, phi, s, "port"), z[f"{nm}/pull"]) <= TOL, nm
        assert rel_err(O.pull_grad(f0, phi, s, "port"), z[f"{nm}/pullg"]) <= TOL, nm
        assert rel_err(O.push(f1, phi, f0.shape[:3], s, "port"), z[f"{nm}/push"]) <= TOL, nm
        if f"{nm}/pushg" in z.files:
            assert rel_err(O.push_grad(g1, phi, f0.shape[:3], s, "port"), z[f"{nm}/pushg"]) <= TOL, nm


def test_oracle_affine_matches_reference(golden, O):
    z, index = golden
    for case in index["affine"]:
        nm = case["name"]
        s = golden_sett(O, case)
        A, f0, f1 = z[f"{nm}/A"], z[f"{nm}/f0"], z[f"{nm}/f1"]
        assert rel_err(O.pull_affine(f0, A, case["d1"], s), z[f"{nm}/pull_affine"]) <= TOL, nm
        assert rel_err(O.push_affine(f1, A, case["d0"], s), z[f"{nm}/push_affine"]) <= TOL, nm


def test_reference_cpu_pushg_defect_is_not_the_contract(O):
    """The reference CPU pushg adds nothing for finite input (artifacts/C/pushpull.c:144);
    the oracle's push_grad is the true adjoint of pull_grad instead."""
    if not O.ref_available():
        pytest.skip("reference sources not present")
    import ctypes as C
    rng = np.random.default_rng(3)
    d0 = (6, 5, 4)
    phi = np.asfortranarray((O.identity(d0) + 0.7 * rng.standard_normal(d0 + (3,))).astype(np.float32))
    g1 = np.asfortranarray(rng.standard_normal(d0 + (3,)).astype(np.float32))
    out = np.zeros(d0, np.float32, order="F")
    so = O.lib("ref")
    n1 = int(np.prod(d0))
    so.pushg(C.c_void_p(out.ctypes.data), C.c_void_p(phi.ctypes.data), C.c_void_p(g1.ctypes.data),
             (C.c_ulonglong * 3)(*d0), C.c_ulonglong(n1), (C.c_int * 3)(1, 1, 1),
             (C.c_ulonglong * 3)(3, 3, 3), C.c_int(1))
    assert not out.any()
    assert np.abs(O.push_grad(g1, phi, d0, O.Sett.make(2, 1, 1))).max() > 0


@pytest.mark.parametrize("deg", [1, 2, 3, 4])
def test_oracle_matches_reference_at_far_coordinates(O, deg):
    """Coordinates of 1e9 (float32 spacing 64): float rounding puts the spline
    offset t on a knot (t = 0 for degree 1), where the derivative weights of
    degree 1 and the second-derivative weights of degree 2 are the reference's
    constants.  The oracle must still agree with the reference library there."""
    if not O.ref_available():
        pytest.skip("reference sources not present")
    rng = np.random.default_rng(400 + deg)
    d = (12, 10, 9)
    f0 = np.asfortranarray(rng.standard_normal(d + (2,)).astype(np.float32))
    phi = (O.identity(d) + 2.0 * rng.standard_normal(d + (3,))).astype(np.float32)
    flat = phi.reshape(-1, order="F")
    flat[rng.choice(flat.size, 60, replace=False)] = 1e9
    phi = np.asfortranarray(phi)
    s = O.Sett.make(deg, 1, 1)
    for op in ("pull", "pull_grad", "pull_hess"):
        a = getattr(O, op)(f0, phi, s)
        b = getattr(O, op)(f0, phi, s, kind="ref")
        assert rel_err(a, b) <= TOL, (deg, op)
