"""Shared fixtures: the host package, the CPU oracle, the golden vectors."""
from __future__ import annotations

import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__ as entry  # noqa: E402

GOLDEN = os.path.join(ROOT, "tests", "golden", "pushpull_golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built native library")
    config.addinivalue_line("markers", "slow: full-size case (seconds of CPU oracle work)")


def pytest_collection_modifyitems(config, items):
    import torch
    if torch.cuda.is_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def pkg():
    return entry.package()


@pytest.fixture(scope="session")
def O():
    from oracle import oracle
    return oracle


@pytest.fixture(scope="session")
def golden():
    z = np.load(GOLDEN)
    index = json.loads(bytes(z["__index__"]).decode())
    return z, index


def rel_err(a, b) -> float:
    """Norm-wise relative error max|a-b| / max|b| over entries where ``b`` is not NaN.

    Also asserts the NaN masks agree exactly."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    assert a.shape == b.shape, (a.shape, b.shape)
    assert (np.isnan(a) == np.isnan(b)).all(), "NaN masks differ"
    m = ~np.isnan(b)
    if not m.any():
        return 0.0
    scale = np.abs(b[m]).max()
    return float(np.abs(a[m] - b[m]).max() / scale) if scale > 0 else float(np.abs(a[m]).max())


def golden_sett(O, case):
    bnd = [tuple(b) for b in case["bnd"]]
    return O.Sett.make(tuple(case["deg"]), bnd if len(bnd) > 1 else bnd[0], case["ext"])


def elem_rel_err(a, b, floor: float = 1e-3) -> float:
    """Elementwise relative error: max |a-b| / |b| over entries with
    |b| > floor * max|b| (NaN masks must agree).  Entries below the floor are
    left to the norm-wise ``rel_err``: a float32 sum whose terms cancel to near
    zero carries an absolute, not a relative, rounding error."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    assert a.shape == b.shape, (a.shape, b.shape)
    assert (np.isnan(a) == np.isnan(b)).all(), "NaN masks differ"
    m = ~np.isnan(b)
    if not m.any():
        return 0.0
    av, bv = a[m], b[m]
    big = np.abs(bv) > floor * np.abs(bv).max()
    if not big.any():
        return 0.0
    return float((np.abs(av[big] - bv[big]) / np.abs(bv[big])).max())


def errors(a, b, floor: float = 1e-3) -> dict:
    """Norm-wise and elementwise relative errors of ``a`` against ``b``."""
    return {"norm": rel_err(a, b), "elem": elem_rel_err(a, b, floor)}
