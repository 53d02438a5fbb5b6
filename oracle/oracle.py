"""ctypes front end of the CPU checkers (test infrastructure only).

Arrays use the reference's Julia layout: numpy arrays in Fortran order with
shapes ``f (d1, d2, d3[, C[, B]])``, ``phi (d1, d2, d3, 3[, B])``,
``grad (d1, d2, d3, 3[, C[, B]])`` and ``hess (d1, d2, d3, 3, 3[, C[, B]])``.
The (batch, channel) loops and the per-channel boundary choice restate
``src/pushpull_cpu.jl:17-259``.

Back ends:
  ``"oracle"``  FP64 restatement (``ora_*``), results in float64.
  ``"port"``    FP32 port with the reference signatures (``port_*``).
  ``"ref"``     the reference's own ``pushpull.c`` compiled from source
                (``_ref/libpp_ref.so``); only where it could be built.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from dataclasses import dataclass

import numpy as np

from . import build as _build

_f32p = np.ctypeslib.ndpointer(np.float32, flags="F_CONTIGUOUS")
_u64p = C.POINTER(C.c_ulonglong)
_i32p = C.POINTER(C.c_int)

_LIBS: dict[str, C.CDLL] = {}
_LOCK = threading.Lock()

# symbol names per back end: (pull, pullg, pullh, push, pushg)
_NAMES = {
    "oracle": dict(pull="ora_pull", pullg="ora_pullg", pullh="ora_pullh",
                   push="ora_push", pushg="ora_pushg",
                   pull_affine="ora_pull_affine", push_affine="ora_push_affine"),
    "port": dict(pull="port_pull", pullg="port_pullg", push="port_push",
                 pushg="port_pushg"),
    # the reference's CPU pushg adds nothing for finite input (pushpull.c:144),
    # so it is not exposed; push_grad parity uses the oracle and the adjoint.
    "ref": dict(pull="pull", pullg="pullg", pullh="pullh", push="push",
                pull_affine="pull_affine", push_affine="push_affine"),
}


@dataclass(frozen=True)
class Sett:
    """Minimal restatement of ``Settings`` (src/pushpull_general.jl:15-60)."""
    deg: tuple
    bnd: tuple  # tuple of 3-tuples, one or one per channel
    ext: int

    @staticmethod
    def make(deg=1, bnd=1, ext=1) -> "Sett":
        if isinstance(deg, (int, np.integer)):
            deg = (deg, deg, deg)
        deg = tuple(int(max(min(d, 4), 0)) for d in deg)
        if isinstance(bnd, (int, np.integer)):
            bnd = ((int(bnd),) * 3,)
        elif len(bnd) == 3 and all(isinstance(b, (int, np.integer)) for b in bnd):
            bnd = (tuple(int(b) for b in bnd),)
        else:
            bnd = tuple(tuple(int(v) for v in b) for b in bnd)
        for b in bnd:
            assert all(v in (0, 1, 2) for v in b)
        return Sett(deg, bnd, int(max(min(int(ext), 1), 0)))

    def bnd_for(self, c: int) -> tuple:
        return self.bnd[0] if len(self.bnd) == 1 else self.bnd[c]


def _as_sett(s) -> Sett:
    if isinstance(s, Sett):
        return s
    return Sett.make(tuple(int(d) for d in s.deg), tuple(tuple(int(v) for v in b) for b in s.bnd),
                     int(s.ext))


def lib(kind: str = "oracle") -> C.CDLL:
    with _LOCK:
        if kind in _LIBS:
            return _LIBS[kind]
        if kind in ("oracle", "port"):
            path = _build.build_oracle()
        elif kind == "ref":
            path = _build.build_ref()
            if path is None or not os.path.exists(path):
                raise RuntimeError("reference library unavailable (reference sources absent)")
        else:
            raise ValueError(kind)
        so = C.CDLL(path)
        for key, sym in _NAMES[kind].items():
            fn = getattr(so, sym)
            fn.restype = C.c_double if sym == "ora_pull_at" else None
        if kind == "oracle":
            so.ora_pull_at.restype = C.c_double
        _LIBS[kind] = so
        return so


def ref_available() -> bool:
    try:
        lib("ref")
        return True
    except Exception:
        return False


def _u64(vals) -> C.Array:
    return (C.c_ulonglong * len(vals))(*[int(v) for v in vals])


def _i32(vals) -> C.Array:
    return (C.c_int * len(vals))(*[int(v) for v in vals])


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def _pad(shape, upto):
    shape = tuple(shape)
    return shape + (1,) * (upto - len(shape))


def _out_dtype(kind):
    return np.float64 if kind == "oracle" else np.float32


def _check_f(a):
    a = np.asarray(a)
    assert a.dtype == np.float32, "inputs are Float32"
    return np.asfortranarray(a)


def pull(f0, phi, sett, kind: str = "oracle", _op: str = "pull", threads: int = 1):
    """f1 = pull(f0, phi) -- src/pushpull_cpu.jl:17-53 (pull_grad :69, pull_hess :111).

    ``threads`` > 1 splits each (batch, channel) call into voxel slabs run in parallel."""
    sett = _as_sett(sett)
    f0, phi = _check_f(f0), _check_f(phi)
    assert 3 <= f0.ndim <= 5 and 4 <= phi.ndim <= 5 and phi.shape[3] == 3
    fs, ps = _pad(f0.shape, 5), _pad(phi.shape, 5)
    assert ps[4] == fs[4]
    nc, nb = fs[3], fs[4]
    assert len(sett.bnd) in (1, nc)
    n0 = fs[0] * fs[1] * fs[2]
    d1 = ps[:3]
    n1 = d1[0] * d1[1] * d1[2]
    ncomp = {"pull": 1, "pullg": 3, "pullh": 9}[_op]
    extra = {"pull": (), "pullg": (3,), "pullh": (3, 3)}[_op]
    out = np.zeros(d1 + extra + tuple(f0.shape[3:]), dtype=_out_dtype(kind), order="F")
    so = lib(kind)
    fn = getattr(so, _NAMES[kind][_op])
    d0 = _u64(fs[:3])
    dp = _u64([d + 1 for d in sett.deg])
    of = out.reshape(-1, order="F")
    ff = f0.reshape(-1, order="F")
    pf = phi.reshape(-1, order="F")
    for b in range(nb):
        for c in range(nc):
            bnd = _i32(sett.bnd_for(c))
            o = of[ncomp * n1 * (nc * b + c):]
            if threads > 1 and n1 >= 4 * threads:
                _pull_slabs(fn, o, pf[3 * n1 * b:3 * n1 * (b + 1)], ff[n0 * (nc * b + c):], d0, n1, ncomp,
                            bnd, dp, sett.ext, threads, out.dtype)
                continue
            fn(_ptr(o), _ptr(pf[3 * n1 * b:]), _ptr(ff[n0 * (nc * b + c):]),
               d0, C.c_ulonglong(n1), bnd, dp, C.c_int(sett.ext))
    return out


def _slabs(n1, threads):
    edges = np.linspace(0, n1, threads + 1).astype(np.int64)
    return [(int(edges[t]), int(edges[t + 1])) for t in range(threads) if edges[t + 1] > edges[t]]


def _planar_slab(flat, n1, comps, a, b):
    """Components [a, b) of a planar (n1, comps) array as a contiguous planar block."""
    return np.ascontiguousarray(flat[:comps * n1].reshape(comps, n1)[:, a:b]).reshape(-1)


def _pull_slabs(fn, o, pf, ff, d0, n1, ncomp, bnd, dp, ext, threads, dtype):
    """One (batch, channel) pull split into contiguous voxel slabs run on a thread
    pool (the C calls release the GIL); each slab gets its own planar copy of its
    deformation, as the reference ABI addresses component k at phi[i + k*n]"""
    from concurrent.futures import ThreadPoolExecutor

    def one(ab):
        a, b = ab
        n = b - a
        ph = _planar_slab(pf, n1, 3, a, b)
        res = np.zeros(ncomp * n, dtype=dtype)
        fn(_ptr(res), _ptr(ph), _ptr(ff), d0, C.c_ulonglong(n), bnd, dp, C.c_int(ext))
        o[:ncomp * n1].reshape(ncomp, n1)[:, a:b] = res.reshape(ncomp, n)

    with ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(one, _slabs(n1, threads)))


def _push_slabs(fn, o, pf, ff, dd, n0, n1, ncomp, bnd, dp, ext, threads, dtype):
    """One (batch, channel) push split into voxel slabs, each scattering into a
    private zeroed image; the private images are summed in slab order."""
    from concurrent.futures import ThreadPoolExecutor

    def one(ab):
        a, b = ab
        n = b - a
        ph = _planar_slab(pf, n1, 3, a, b)
        vals = _planar_slab(ff, n1, ncomp, a, b)
        acc = np.zeros(n0, dtype=dtype)
        fn(_ptr(acc), _ptr(ph), _ptr(vals), dd, C.c_ulonglong(n), bnd, dp, C.c_int(ext))
        return acc

    with ThreadPoolExecutor(max_workers=threads) as ex:
        parts = list(ex.map(one, _slabs(n1, threads)))
    for acc in parts:
        o[:n0] += acc


def pull_grad(f0, phi, sett, kind: str = "oracle", threads: int = 1):
    return pull(f0, phi, sett, kind, "pullg", threads)


def pull_hess(f0, phi, sett, kind: str = "oracle", threads: int = 1):
    return pull(f0, phi, sett, kind, "pullh", threads)


def push(f1, phi, d0, sett, kind: str = "oracle", _op: str = "push", threads: int = 1):
    """f0 = push(f1, phi, d0) -- src/pushpull_cpu.jl:165-203 (push_grad :220-259).

    ``threads`` > 1 splits each (batch, channel) call into voxel slabs run in parallel."""
    sett = _as_sett(sett)
    f1, phi = _check_f(f1), _check_f(phi)
    grad = _op == "pushg"
    lead = 4 if grad else 3
    if grad:
        assert f1.shape[3] == 3
    fs = _pad(f1.shape, lead + 2)
    ps = _pad(phi.shape, 5)
    assert fs[:3] == ps[:3] and ps[3] == 3 and ps[4] == fs[lead + 1]
    nc, nb = fs[lead], fs[lead + 1]
    assert len(sett.bnd) in (1, nc)
    d0 = tuple(int(v) for v in d0)
    n0 = d0[0] * d0[1] * d0[2]
    n1 = ps[0] * ps[1] * ps[2]
    ncomp = 3 if grad else 1
    out = np.zeros(d0 + tuple(f1.shape[lead:]), dtype=_out_dtype(kind), order="F")
    so = lib(kind)
    fn = getattr(so, _NAMES[kind][_op])
    dd = _u64(d0)
    dp = _u64([d + 1 for d in sett.deg])
    of = out.reshape(-1, order="F")
    ff = f1.reshape(-1, order="F")
    pf = phi.reshape(-1, order="F")
    for b in range(nb):
        for c in range(nc):
            bnd = _i32(sett.bnd_for(c))
            if threads > 1 and n1 >= 4 * threads:
                _push_slabs(fn, of[n0 * (nc * b + c):n0 * (nc * b + c + 1)], pf[3 * n1 * b:3 * n1 * (b + 1)],
                            ff[ncomp * n1 * (nc * b + c):], dd, n0, n1, ncomp, bnd, dp, sett.ext, threads,
                            out.dtype)
                continue
            fn(_ptr(of[n0 * (nc * b + c):]), _ptr(pf[3 * n1 * b:]),
               _ptr(ff[ncomp * n1 * (nc * b + c):]),
               dd, C.c_ulonglong(n1), bnd, dp, C.c_int(sett.ext))
    return out


def push_grad(g1, phi, d0, sett, kind: str = "oracle", threads: int = 1):
    return push(g1, phi, d0, sett, kind, "pushg", threads)


def adjust_affine(A):
    """3x4 (or 4x4) 1-based affine -> 0-based, src/pushpull_cpu.jl:357-362."""
    A = np.asarray(A, dtype=np.float32)
    assert A.shape[1] == 4 and A.shape[0] in (3, 4)
    B = A[:3, :].astype(np.float32).copy()
    B[:, 3] = (B.sum(axis=1) - np.float32(1.0)).astype(np.float32)
    return B


def pull_affine(f0, A, d1, sett, kind: str = "oracle"):
    """src/pushpull_cpu.jl:268-307 with the reference C at pushpull.c:176-209."""
    sett = _as_sett(sett)
    f0 = _check_f(f0)
    B = np.asfortranarray(adjust_affine(A))
    fs = _pad(f0.shape, 5)
    nc, nb = fs[3], fs[4]
    d1 = tuple(int(v) for v in d1)
    n0 = fs[0] * fs[1] * fs[2]
    n1 = d1[0] * d1[1] * d1[2]
    out = np.zeros(d1 + tuple(f0.shape[3:]), dtype=_out_dtype(kind), order="F")
    fn = getattr(lib(kind), _NAMES[kind]["pull_affine"])
    of, ff = out.reshape(-1, order="F"), f0.reshape(-1, order="F")
    for b in range(nb):
        for c in range(nc):
            fn(_ptr(of[n1 * (nc * b + c):]), _ptr(ff[n0 * (nc * b + c):]), _u64(fs[:3]),
               C.c_ulonglong(n1), _u64(d1), _ptr(B), _i32(sett.bnd_for(c)),
               _u64([d + 1 for d in sett.deg]), C.c_int(sett.ext))
    return out


def push_affine(f1, A, d0, sett, kind: str = "oracle"):
    """src/pushpull_cpu.jl:310-349 with the reference C at pushpull.c:213-244."""
    sett = _as_sett(sett)
    f1 = _check_f(f1)
    B = np.asfortranarray(adjust_affine(A))
    fs = _pad(f1.shape, 5)
    nc, nb = fs[3], fs[4]
    d0 = tuple(int(v) for v in d0)
    n0 = d0[0] * d0[1] * d0[2]
    n1 = fs[0] * fs[1] * fs[2]
    out = np.zeros(d0 + tuple(f1.shape[3:]), dtype=_out_dtype(kind), order="F")
    fn = getattr(lib(kind), _NAMES[kind]["push_affine"])
    of, ff = out.reshape(-1, order="F"), f1.reshape(-1, order="F")
    for b in range(nb):
        for c in range(nc):
            fn(_ptr(of[n0 * (nc * b + c):]), _ptr(ff[n1 * (nc * b + c):]), _u64(d0),
               C.c_ulonglong(n1), _u64(fs[:3]), _ptr(B), _i32(sett.bnd_for(c)),
               _u64([d + 1 for d in sett.deg]), C.c_int(sett.ext))
    return out


def pull_at(pos, f0, sett, c: int = 0) -> float:
    """FP64 pull of one channel of a 3-D volume at one 1-based float32 position."""
    sett = _as_sett(sett)
    f0 = _check_f(f0)
    fs = _pad(f0.shape, 5)
    n0 = fs[0] * fs[1] * fs[2]
    p = (C.c_float * 3)(*[float(np.float32(v)) for v in pos])
    so = lib("oracle")
    ff = f0.reshape(-1, order="F")
    return so.ora_pull_at(p, _ptr(ff[n0 * c:]), _u64(fs[:3]), _i32(sett.bnd_for(c)),
                          _u64([d + 1 for d in sett.deg]), C.c_int(sett.ext))


def identity(d, affine=None) -> np.ndarray:
    """1-based identity deformation (d1, d2, d3, 3), src/pushpull_general.jl:81-99."""
    x = np.arange(1, d[0] + 1, dtype=np.float32)[:, None, None]
    y = np.arange(1, d[1] + 1, dtype=np.float32)[None, :, None]
    z = np.arange(1, d[2] + 1, dtype=np.float32)[None, None, :]
    phi = np.zeros(tuple(d) + (3,), dtype=np.float32, order="F")
    if affine is None:
        phi[..., 0] = x
        phi[..., 1] = y
        phi[..., 2] = z
    else:
        A = np.asarray(affine, dtype=np.float64)
        for k in range(3):
            phi[..., k] = (A[k, 0] * x + A[k, 1] * y + A[k, 2] * z + A[k, 3]).astype(np.float32)
    return phi
