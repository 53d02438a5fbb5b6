"""Batched uneven workload: many (image, deformation) pairs -- e.g. registration
pairs and their multigrid pyramid levels -- pulled (f1 = pull(f0, phi)) and
pushed back (out += push(f1, phi)) in one persistent launch, optionally
replayed from a CUDA graph (include/pushpull_gb300.h, pp_batch_*)."""
from __future__ import annotations

import ctypes as C

import torch

from . import _native
from . import layout as L
from .settings import Settings


class BatchPlan:
    """``items``: dicts with ``f0 (d0[, C])``, ``phi (d1, 3)``, ``f1 (d1[, C])``,
    ``out (d0[, C])`` (column-major CUDA float32 tensors) and ``sett`` (any
    per-dimension degrees; one boundary triple, or one per channel)."""

    def __init__(self, items, zero_outputs: bool = True):
        self._lib = _native.lib()
        self._keep = []
        arr = (_native.BatchItem * len(items))()
        for i, it in enumerate(items):
            f0, phi, f1, out = (L.colmajor(it[k]) for k in ("f0", "phi", "f1", "out"))
            for t in (f0, phi, f1, out):
                if t.device.type != "cuda" or t.dtype != torch.float32:
                    raise TypeError("batch arrays must be CUDA float32 tensors")
            s: Settings = it["sett"]
            nc = L.jsize(f0, 4)
            assert len(s.bnd) in (1, nc), "one boundary triple, or one per channel"
            self._keep += [f0, phi, f1, out]
            e = arr[i]
            e.f0, e.phi, e.f1, e.out = f0.data_ptr(), phi.data_ptr(), f1.data_ptr(), out.data_ptr()
            e.d0 = (C.c_ulonglong * 3)(*f0.shape[:3])
            e.d1 = (C.c_ulonglong * 3)(*phi.shape[:3])
            iso = s.deg[0] == s.deg[1] == s.deg[2]
            e.nc, e.deg, e.ext = nc, s.deg[0] if iso else -1, s.ext
            e.deg3 = (C.c_int * 3)(*s.deg)
            e.bnd = (C.c_int * 3)(*s.bnd[0])
            if len(s.bnd) > 1:
                codes = (C.c_int * (3 * nc))(*[v for b in s.bnd for v in b])   # read by pp_batch_create
                self._keep.append(codes)
                e.nbnd, e.bnds = nc, C.cast(codes, C.c_void_p)
        self._h = C.c_void_p()
        _native.check("pp_batch_create", self._lib.pp_batch_create(C.byref(self._h), arr, len(items),
                                                                    int(bool(zero_outputs))))

    @property
    def tiles(self) -> int:
        return self._lib.pp_batch_tiles(self._h)

    def _stream(self, stream):
        return (stream or torch.cuda.current_stream()).cuda_stream

    def run(self, stream=None):
        _native.check("pp_batch_run", self._lib.pp_batch_run(self._h, self._stream(stream)))

    def capture(self, stream=None):
        _native.check("pp_batch_capture", self._lib.pp_batch_capture(self._h, self._stream(stream)))

    def launch(self, stream=None):
        _native.check("pp_batch_launch", self._lib.pp_batch_launch(self._h, self._stream(stream)))

    def close(self):
        if getattr(self, "_h", None):
            self._lib.pp_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
