"""Batched uneven workload (pp_batch_*): every item of one persistent launch
matches the single-array pull / push of that item (pull bit-identical, push
1e-4 norm-wise relative), one item is checked against the FP64 oracle, and the
CUDA-graph replay reproduces the eager run."""
from __future__ import annotations

import importlib

import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _items(pkg, W, specs):
    L = pkg.layout
    items = []
    for k, (d, nc, deg, bnd, ext) in enumerate(specs):
        f0 = W.image_gpu(d, 100 + k, fwhm=3.0, channels=nc)
        phi = W.deformation_gpu(d, 200 + k, fwhm=8.0, amplitude=2.5)
        f1 = L.empty(d + ((nc,) if nc > 1 else ()))
        out = L.empty(tuple(f0.shape))
        items.append(dict(f0=f0, phi=phi, f1=f1, out=out, sett=pkg.Settings(deg, bnd, ext)))
    return items


SPECS = [((40, 33, 29), 2, 3, 1, 1), ((20, 17, 15), 2, 3, 1, 1), ((10, 9, 8), 2, 3, 1, 1),
         ((36, 28, 24), 1, 1, 0, 0), ((18, 14, 12), 1, 1, 0, 0), ((33, 31, 17), 3, 2, (0, 1, 2), 1),
         ((17, 16, 9), 3, 2, (0, 1, 2), 1), ((64, 8, 4), 1, 4, 2, 1)]


def test_batch_matches_single_calls(pkg, O):
    W = importlib.import_module("pushpull_gb300.workloads")
    B = importlib.import_module("pushpull_gb300.batch")
    L = pkg.layout
    items = _items(pkg, W, SPECS)
    plan = B.BatchPlan(items, zero_outputs=True)
    assert plan.tiles > 0
    plan.run()
    torch.cuda.synchronize()
    for it in items:
        s = it["sett"]
        ref1 = pkg.pull(it["f0"], it["phi"], s)
        ref0 = pkg.push(ref1, it["phi"], tuple(it["f0"].shape[:3]), s)
        assert torch.equal(torch.isnan(it["f1"]), torch.isnan(ref1))
        assert rel_err(L.to_numpy(it["f1"]), L.to_numpy(ref1)) <= 1e-6
        assert rel_err(L.to_numpy(it["out"]), L.to_numpy(ref0)) <= 1e-4
    # one item against the FP64 oracle
    it = items[5]
    f0, phi = L.to_numpy(it["f0"]), L.to_numpy(it["phi"])
    so = O.Sett.make(2, (0, 1, 2), 1)
    ref1 = O.pull(f0, phi, so)
    assert rel_err(L.to_numpy(it["f1"]), ref1) <= 1e-5
    assert rel_err(L.to_numpy(it["out"]), O.push(L.to_numpy(it["f1"]), phi, f0.shape[:3], so)) <= 1e-4
    plan.close()


def test_batch_graph_replay(pkg):
    W = importlib.import_module("pushpull_gb300.workloads")
    B = importlib.import_module("pushpull_gb300.batch")
    items = _items(pkg, W, SPECS[:5])
    plan = B.BatchPlan(items, zero_outputs=True)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        plan.run(stream)
    stream.synchronize()
    first = [it["out"].clone() for it in items]
    with torch.cuda.stream(stream):
        plan.capture(stream)
        for _ in range(3):
            plan.launch(stream)
    stream.synchronize()
    for it, ref in zip(items, first):
        assert (it["out"] - ref).abs().max() <= 1e-4 * ref.abs().max()
    assert pkg.native_library().pp_device_status(1) == 0
    plan.close()


def test_batch_general_items(pkg, O):
    """Items with per-dimension degrees and per-channel boundary triples, mixed
    with isotropic ones, in one plan: each against its single calls and the FP64
    oracle."""
    W = importlib.import_module("pushpull_gb300.workloads")
    B = importlib.import_module("pushpull_gb300.batch")
    L = pkg.layout
    specs = [((30, 26, 22), 2, (1, 3, 2), [(0, 1, 2), (1, 1, 1)], 1),
             ((24, 20, 28), 3, 3, [(1, 1, 1), (2, 2, 2), (0, 0, 0)], 1),
             ((20, 18, 16), 1, (3, 0, 4), 1, 0),
             ((32, 24, 16), 2, 2, (0, 1, 2), 1)]
    items = _items(pkg, W, specs)
    plan = B.BatchPlan(items, zero_outputs=True)
    plan.run()
    torch.cuda.synchronize()
    assert pkg.native_library().pp_device_status(1) == 0
    for it, (d, nc, deg, bnd, ext) in zip(items, specs):
        s = it["sett"]
        ref1 = pkg.pull(it["f0"], it["phi"], s)
        ref0 = pkg.push(ref1, it["phi"], d, s)
        assert torch.equal(torch.isnan(it["f1"]), torch.isnan(ref1))
        assert rel_err(L.to_numpy(it["f1"]), L.to_numpy(ref1)) <= 1e-5
        assert rel_err(L.to_numpy(it["out"]), L.to_numpy(ref0)) <= 1e-4
        so = O.Sett.make(deg, bnd, ext)
        f0, phi, f1 = L.to_numpy(it["f0"]), L.to_numpy(it["phi"]), L.to_numpy(it["f1"])
        assert rel_err(f1, O.pull(f0, phi, so)) <= 1e-5
        assert rel_err(L.to_numpy(it["out"]), O.push(f1, phi, d, so)) <= 1e-4
    plan.close()
