"""Timed CPU baseline of pull + push (test/benchmark infrastructure only).

Runs the reference's CPU library compiled from source (``kind="reference"``,
only where it could be built) or the FP32 port with the same signatures
(``kind="port"``) over all host threads:

* pull: the sample voxels are split into contiguous slabs, one per thread; each
  thread gets its own contiguous copy of its slab of the deformation (made
  before timing) because the reference ABI addresses component k at
  ``phi[i + k*n1]`` of the slab it is given;
* push: the same slabs, each thread scattering into a private zeroed
  accumulator; the accumulators are then summed (timed).

The reference library is single threaded (its OpenMP pragma is commented out,
artifacts/C/pushpull.c:18-20); this harness only runs independent calls in
parallel, as a user would.
"""
from __future__ import annotations

import ctypes as C
import os
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import oracle as O


class PullPushCPU:
    def __init__(self, f0, phi, deg, bnd, ext, threads=None, kind=None):
        if kind is None:
            kind = "reference" if O.ref_available() else "port"
        self.kind = kind
        so = O.lib("ref" if kind == "reference" else "port")
        self.pull_fn = so.pull if kind == "reference" else so.port_pull
        self.push_fn = so.push if kind == "reference" else so.port_push
        self.threads = int(threads or os.cpu_count() or 1)
        self.f0 = np.asfortranarray(f0, dtype=np.float32)
        self.d0 = tuple(int(v) for v in f0.shape[:3])
        self.n0 = int(np.prod(self.d0))
        d1 = phi.shape[:3]
        self.n1 = int(np.prod(d1))
        flat = np.asarray(phi, dtype=np.float32).reshape((self.n1, 3), order="F")
        bounds = np.linspace(0, self.n1, self.threads + 1).astype(np.int64)
        self.slabs = []
        for t in range(self.threads):
            a, b = int(bounds[t]), int(bounds[t + 1])
            self.slabs.append((a, b, np.asfortranarray(flat[a:b, :].copy(order="F"))))
        self.f1 = np.zeros(self.n1, dtype=np.float32)
        self.acc = [np.zeros(self.n0, dtype=np.float32) for _ in range(self.threads)]
        self.out = np.zeros(self.n0, dtype=np.float32)
        self.c_d0 = (C.c_ulonglong * 3)(*self.d0)
        bnd = bnd if isinstance(bnd, (tuple, list)) else (bnd,) * 3
        self.c_bnd = (C.c_int * 3)(*[int(v) for v in bnd])
        self.c_dp = (C.c_ulonglong * 3)(*[int(d) + 1 for d in deg])
        self.ext = int(ext)
        self.pool = ThreadPoolExecutor(max_workers=self.threads)

    def _pull(self, t):
        a, b, ph = self.slabs[t]
        if b <= a:
            return
        self.pull_fn(C.c_void_p(self.f1.ctypes.data + 4 * a), C.c_void_p(ph.ctypes.data),
                     C.c_void_p(self.f0.ctypes.data), self.c_d0, C.c_ulonglong(b - a), self.c_bnd,
                     self.c_dp, C.c_int(self.ext))

    def _push(self, t):
        a, b, ph = self.slabs[t]
        acc = self.acc[t]
        acc.fill(0.0)
        if b <= a:
            return
        self.push_fn(C.c_void_p(acc.ctypes.data), C.c_void_p(ph.ctypes.data),
                     C.c_void_p(self.f1.ctypes.data + 4 * a), self.c_d0, C.c_ulonglong(b - a),
                     self.c_bnd, self.c_dp, C.c_int(self.ext))

    def step(self) -> float:
        """One pull of the whole sample grid then one push of the result; returns seconds."""
        t0 = time.perf_counter()
        list(self.pool.map(self._pull, range(self.threads)))
        list(self.pool.map(self._push, range(self.threads)))
        np.copyto(self.out, self.acc[0])
        for a in self.acc[1:]:
            self.out += a
        return time.perf_counter() - t0

    def close(self):
        self.pool.shutdown()
