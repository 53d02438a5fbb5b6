"""Every benchmark workload at its full size, through the C ABI, against the FP64
oracle (and, where it was built, the reference's own CPU library).

* C1  64^3, trilinear, circulant, ext = 0: pull, pull_grad, push, push_grad on
      both kernel families (the per-voxel default and the tiled kernels forced
      with pp_set_tile).
* C2  192^3, cubic, DCT-II, ext = 1: pull_grad against FP64; pull and push
      against the reference library compiled from its sources.
* C3  160x192x160, quadratic, bounds (0,1,2): the fused step's deformation
      gradient against central finite differences (h = 1e-3 vox, FP64 point
      evaluations) at 64 seeded voxels, all three components.
* C4  the full uneven batch (32 pairs x 3 pyramid levels): every item of the
      persistent plan against its own single calls, and one item per degree
      against FP64.
* C5  256^3 x 3 channels, cubic, 0.25x contraction: the adjoint identity
      <pull_grad(b), G> = <b, push_grad(G)> in float64 sums.

Tolerances: values (pull, and push of non-negative data) within 1e-5 (pull) or
1e-4 (push) both norm-wise (max|a-b| / max|b|) and elementwise over entries
above 1e-3 of the largest.  Derivatives (pull_grad, push_grad of signed data,
the deformation gradient) are sums whose terms cancel, so their float32 rounding
is absolute rather than relative: norm-wise within 1e-4, elementwise within
1e-3 over entries above 1e-2 of the largest.
"""
from __future__ import annotations

import ctypes as C
import importlib
import os

import numpy as np
import pytest
import torch

from conftest import elem_rel_err, rel_err

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

THREADS = max(1, min(16, os.cpu_count() or 1))


@pytest.fixture(scope="module")
def W(pkg):
    return importlib.import_module("pushpull_gb300.workloads")


def _value_ok(got, ref, tol, what):
    e_n, e_e = rel_err(got, ref), elem_rel_err(got, ref, 1e-3)
    print(f"{what}: norm {e_n:.2e} elem {e_e:.2e}")
    assert e_n <= tol and e_e <= tol, (what, e_n, e_e)


def _deriv_ok(got, ref, what):
    e_n, e_e = rel_err(got, ref), elem_rel_err(got, ref, 1e-2)
    print(f"{what}: norm {e_n:.2e} elem(1e-2) {e_e:.2e}")
    assert e_n <= 1e-4 and e_e <= 1e-3, (what, e_n, e_e)


@pytest.fixture
def tiles(pkg):
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


@pytest.mark.parametrize("family", ["default", "tiled", "direct"])
def test_c1_all_ops_vs_oracle(pkg, O, W, tiles, family):
    """The 64^3 trilinear workload on each kernel family: the defaults
    (warp-specialised pull and pull_grad, per-voxel push), the block-synchronous
    tiled kernels, and the per-voxel kernels for every op."""
    L = pkg.layout
    w = W.config1()
    if family == "tiled":
        for op, cap in ((0, 8192), (1, 8192), (3, 16384), (4, 16384)):
            assert tiles.pp_set_tile(op, 1, 3, 3, 3, cap) == 0
    elif family == "direct":
        assert tiles.pp_set_path(1) == 0
    s, so = pkg.Settings(w.deg, w.bnd, w.ext), O.Sett.make(w.deg, w.bnd, w.ext)
    d = w.f0.shape[:3]
    f1 = np.asfortranarray(W.image(d, 11))
    g1 = np.asfortranarray(np.random.default_rng(12).standard_normal(d + (3,)).astype(np.float32))
    tf0, tphi, tf1, tg1 = (L.from_numpy(a) for a in (w.f0, w.phi, f1, g1))
    got = {"pull": pkg.pull(tf0, tphi, s), "pullg": pkg.pull_grad(tf0, tphi, s),
           "push": pkg.push(tf1, tphi, d, s), "pushg": pkg.push_grad(tg1, tphi, d, s)}
    torch.cuda.synchronize()
    got = {k: L.to_numpy(v) for k, v in got.items()}
    assert np.isnan(got["pull"]).any(), "ext = 0 with +-2 vox must leave some samples outside the band"
    _value_ok(got["pull"], O.pull(w.f0, w.phi, so, threads=THREADS), 1e-5, f"C1 {family} pull")
    _deriv_ok(got["pullg"], O.pull_grad(w.f0, w.phi, so, threads=THREADS), f"C1 {family} pull_grad")
    _value_ok(got["push"], O.push(f1, w.phi, d, so, threads=THREADS), 1e-4, f"C1 {family} push")
    _deriv_ok(got["pushg"], O.push_grad(g1, w.phi, d, so, threads=THREADS), f"C1 {family} push_grad")
    assert pkg.native_library().pp_device_status(1) == 0


def test_c2_pull_grad_vs_oracle(pkg, O, W):
    L = pkg.layout
    w = W.config2()
    s, so = pkg.Settings(w.deg, w.bnd, w.ext), O.Sett.make(w.deg, w.bnd, w.ext)
    got = L.to_numpy(pkg.pull_grad(L.from_numpy(w.f0), L.from_numpy(w.phi), s))
    _deriv_ok(got, O.pull_grad(w.f0, w.phi, so, threads=THREADS), "C2 pull_grad")


def test_c2_pull_push_vs_reference_library(pkg, O, W):
    """The benchmark step against the reference's own CPU pull / push (FP32,
    compiled from its sources): the two float32 implementations agree to the
    same tolerances as against FP64."""
    if not O.ref_available():
        pytest.skip("reference library not built on this host")
    L = pkg.layout
    w = W.config2()
    s, so = pkg.Settings(w.deg, w.bnd, w.ext), O.Sett.make(w.deg, w.bnd, w.ext)
    d = w.f0.shape[:3]
    tphi = L.from_numpy(w.phi)
    f1 = L.to_numpy(pkg.pull(L.from_numpy(w.f0), tphi, s))
    ref_f1 = O.pull(w.f0, w.phi, so, kind="ref", threads=THREADS)
    _value_ok(f1, ref_f1, 1e-5, "C2 pull vs reference")
    back = L.to_numpy(pkg.push(L.from_numpy(ref_f1), tphi, d, s))
    _value_ok(back, O.push(ref_f1, w.phi, d, so, kind="ref", threads=THREADS), 1e-4, "C2 push vs reference")


def test_c3_fused_step_finite_differences(pkg, O, W):
    """d loss / d phi of the fused step at 64 seeded sample voxels (all three
    components) against central differences of the FP64 loss, h = 1e-3 vox.
    Only voxel v's own term of the loss depends on phi[v], so each difference
    needs two point evaluations."""
    L = pkg.layout
    w = W.config3()
    s, so = pkg.Settings(w.deg, w.bnd, w.ext), O.Sett.make(w.deg, w.bnd, w.ext)
    g = np.asfortranarray(O.pull(w.f0, w.extra["phi2"], so, threads=THREADS).astype(np.float32))
    loss, df, dphi = pkg.fused_step(L.from_numpy(w.f0), L.from_numpy(w.phi), L.from_numpy(g), s)
    dphi = L.to_numpy(dphi)
    d1 = w.phi.shape[:3]
    rng = np.random.default_rng(33)
    vox = rng.integers(0, int(np.prod(d1)), 64)
    h = 1e-3
    got, fd = [], []
    for v in vox:
        idx = np.unravel_index(int(v), d1, order="F")
        p0 = w.phi[idx].astype(np.float32)
        for k in range(3):
            pp, pm = p0.copy(), p0.copy()
            pp[k] = np.float32(p0[k] + h)
            pm[k] = np.float32(p0[k] - h)
            lp = (O.pull_at(pp, w.f0, so) - float(g[idx])) ** 2
            lm = (O.pull_at(pm, w.f0, so) - float(g[idx])) ** 2
            fd.append((lp - lm) / (float(pp[k]) - float(pm[k])))
            got.append(float(dphi[idx + (k,)]))
    got, fd = np.array(got), np.array(fd)
    crit = float(np.sum((got - fd) ** 2) / np.sum(fd ** 2))   # test/utils.jl:24 criterion, < 1e-3 there
    e = rel_err(got, fd)
    print(f"C3 FD: norm {e:.2e}, sum-of-squares criterion {crit:.2e}")
    assert e <= 1e-3 and crit <= 1e-6, (e, crit)


def test_c4_full_batch_vs_single_calls_and_oracle(pkg, O):
    from pushpull_gb300 import batch as B
    from pushpull_gb300 import workloads as Wl
    L = pkg.layout
    specs = Wl.batched_pairs(seed=4, npairs=32, levels=3)
    items = []
    for sp in specs:
        d, c = sp["d"], sp["channels"]
        f0 = Wl.image_gpu(d, sp["seed"], fwhm=3.0, channels=c)
        phi = Wl.deformation_gpu(d, sp["seed"] + 7, fwhm=8.0, amplitude=3.0 / (1 << sp["level"]))
        shape = tuple(d) + ((c,) if c > 1 else ())
        items.append(dict(f0=f0, phi=phi, f1=L.empty(shape), out=L.empty(shape), sett=pkg.Settings(sp["deg"], 1, 1),
                          spec=sp))
    plan = B.BatchPlan([{k: it[k] for k in ("f0", "phi", "f1", "out", "sett")} for it in items])
    stream = torch.cuda.Stream()
    stream.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(stream):
        plan.capture(stream)
        plan.launch(stream)
    torch.cuda.current_stream().wait_stream(stream)
    torch.cuda.synchronize()
    worst = {"pull": 0.0, "push": 0.0}
    for it in items:
        d0 = tuple(it["f0"].shape[:3])
        f1 = pkg.pull(it["f0"], it["phi"], it["sett"])
        back = pkg.push(it["f1"], it["phi"], d0, it["sett"])
        a, b = L.to_numpy(it["f1"]), L.to_numpy(f1)
        e = max(rel_err(a, b), elem_rel_err(a, b))
        assert e <= 1e-5, (it["spec"], "pull", e)
        a, b = L.to_numpy(it["out"]), L.to_numpy(back)
        e2 = max(rel_err(a, b), elem_rel_err(a, b))
        assert e2 <= 1e-4, (it["spec"], "push", e2)
        worst["pull"], worst["push"] = max(worst["pull"], e), max(worst["push"], e2)
    print("C4 batch vs single calls:", worst)
    for deg in (1, 2, 3):
        it = min((x for x in items if x["spec"]["deg"] == deg), key=lambda x: x["f0"].numel())
        so = O.Sett.make(deg, 1, 1)
        f0, phi = L.to_numpy(it["f0"]), L.to_numpy(it["phi"])
        _value_ok(L.to_numpy(it["f1"]), O.pull(f0, phi, so, threads=THREADS), 1e-5, f"C4 deg {deg} pull")
        f1 = L.to_numpy(it["f1"])
        _value_ok(L.to_numpy(it["out"]), O.push(f1, phi, f0.shape[:3], so, threads=THREADS), 1e-4,
                  f"C4 deg {deg} push")
    plan.close()


def test_c5_push_grad_adjoint_full_size(pkg, W):
    L = pkg.layout
    d = (256, 256, 256)
    s = pkg.Settings(3, 1, 1)
    b = W.image_gpu(d, 71, channels=3)
    G = L.empty(d + (3, 3))
    G.copy_(torch.randn(G.shape, generator=torch.Generator(device="cuda").manual_seed(72), device="cuda"))
    phi = W.deformation_gpu(d, 73, 12.0, 3.0, contraction=0.25)
    pg = pkg.pull_grad(b, phi, s)
    terms = pg.double() * G.double()
    lhs = float(terms.sum())
    scale = float(terms.abs().sum())
    del terms, pg
    rhs = float((b.double() * pkg.push_grad(G, phi, d, s).double()).sum())
    print(f"C5 push_grad adjoint: |lhs-rhs| {abs(lhs - rhs):.3e}, |lhs| {abs(lhs):.3e}, sum|terms| {scale:.3e}")
    assert abs(lhs - rhs) <= 1e-7 * scale and abs(lhs - rhs) <= 1e-5 * abs(lhs)
