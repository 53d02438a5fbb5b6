"""Tile autotuning with a persistent cache.

``tune(op, x, phi, sett, d0=None)`` runs the native autotuner (pp_autotune:
per-voxel kernels and every candidate tile shape / shared-memory budget timed on
these very arrays), installs the winner for (op, degree) and records it in a
JSON cache keyed by device name, op, degree and size class (log2 of the sample
count).  ``load()`` re-installs cached choices in a new process.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os

import torch

from . import _native
from . import layout as L
from .settings import Settings

OPS = {"pull": 0, "pull_grad": 1, "pull_hess": 2, "push": 3, "push_grad": 4}
CACHE = os.environ.get("PUSHPULL_GB300_TUNE_CACHE",
                       os.path.join(os.path.expanduser("~"), ".cache", "pushpull_gb300", "tiles.json"))


def _key(op: str, deg: int, n1: int) -> str:
    dev = torch.cuda.get_device_name()
    return f"{dev}|{op}|deg{deg}|n2^{int(round(math.log2(max(n1, 1))))}"


def _read():
    try:
        with open(CACHE) as fh:
            return json.load(fh)
    except Exception:
        return {}


def tune(op: str, x: torch.Tensor, phi: torch.Tensor, sett: Settings, d0=None, reps: int = 3) -> dict:
    """x: the op's input (image for pull ops, values for push ops)."""
    lib = _native.lib()
    code = OPS[op]
    x, phi = L.colmajor(x), L.colmajor(phi)
    d1 = tuple(phi.shape[:3])
    if code < 3:
        d0 = tuple(x.shape[:3])
        lead = 3
        extra = {0: (), 1: (3,), 2: (3, 3)}[code]
        out = L.empty(d1 + extra + tuple(x.shape[3:]), device=x.device)
    else:
        lead = 4 if code == 4 else 3
        out = L.empty(tuple(d0) + tuple(x.shape[lead:]), device=x.device)
    nc, nb = L.jsize(x, lead + 1), L.jsize(x, lead + 2)
    best = (C.c_int * 5)()
    ms = C.c_float()
    rc = lib.pp_autotune(code, out.data_ptr(), phi.data_ptr(), x.data_ptr(), _native.u64x3(d0), _native.u64x3(d1),
                         nc, nb, sett.bnd_array(), sett.nbnd, _native.i32x3(sett.deg), sett.ext, reps,
                         torch.cuda.current_stream().cuda_stream, best, C.byref(ms))
    _native.check("pp_autotune", rc)
    res = {"tile": [best[0], best[1], best[2]], "cap": best[3], "path": "direct" if best[4] == 1 else "tiled",
           "ms": ms.value}
    cache = _read()
    cache[_key(op, sett.deg[0], int(torch.tensor(d1).prod()))] = res
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    with open(CACHE, "w") as fh:
        json.dump(cache, fh, indent=1, sort_keys=True)
    return res


def load() -> int:
    """Install every cached choice of this device; returns how many."""
    lib = _native.lib()
    dev = torch.cuda.get_device_name()
    n = 0
    for key, res in _read().items():
        d, op, deg, _ = key.split("|")
        if d != dev:
            continue
        lx, ly, lz = res["tile"]
        cap = res["cap"] if res.get("path") == "tiled" else 0     # cap 0: per-voxel kernels
        if lib.pp_set_tile(OPS[op], int(deg[3:]), lx, ly, lz, cap) == 0:
            n += 1
    return n
