"""User API: ``pull``, ``pull_grad``, ``pull_hess``, ``push``, ``push_grad``, ``id``.

Mirrors the reference's host functions (src/pushpull_cpu.jl:17-259 and the
CUDA.jl methods in ext/pushpull_gpu.jl:15-259): same names, argument order,
assertions and messages, Julia shapes and Float32 semantics.  Arrays are
CUDA ``torch.float32`` tensors in column-major layout (see ``layout``); each
call hands the whole (channel, batch) set to one native call on the current
stream.  There is no CPU path: CPU tensors are rejected.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _native
from . import layout as L
from .settings import Settings


def _stream(t: torch.Tensor) -> int:
    return torch.cuda.current_stream(t.device).cuda_stream


def _require_cuda(*ts):
    dev = None
    for t in ts:
        if not isinstance(t, torch.Tensor) or t.device.type != "cuda":
            raise TypeError("pushpull_gb300 operates on CUDA tensors (no CPU path)")
        if t.dtype != torch.float32:
            raise TypeError("arrays must be Float32")
        if dev is None:
            dev = t.device
        elif t.device != dev:
            raise ValueError("all arrays must be on the same device")
    return dev


def _pull_family(fn: str, f0, phi, sett: Settings, ncomp_shape, out=None):
    assert 3 <= f0.dim() <= 5, "`f₀` must have between 3 & 5 dimensions"
    assert 4 <= phi.dim() <= 5, "`ϕ` must have 4 or 5 dimensions"
    assert L.jsize(phi, 4) == 3, "`ϕ` must have three channels"
    assert L.jsize(phi, 5) == L.jsize(f0, 5), "`ϕ` & `f₀` must have the same batch size"
    assert len(sett.bnd) == L.jsize(f0, 4) or len(sett.bnd) == 1
    _require_cuda(f0, phi)
    f0, phi = L.colmajor(f0), L.colmajor(phi)
    nc, nb = L.jsize(f0, 4), L.jsize(f0, 5)
    d0 = tuple(f0.shape[:3])
    d1 = tuple(phi.shape[:3])
    shape = d1 + ncomp_shape + tuple(f0.shape[3:])
    if out is None:
        out = L.empty(shape, device=f0.device)
    else:
        _require_cuda(out)
        assert tuple(out.shape) == shape and L.is_colmajor(out)
    lib = _native.lib()
    rc = getattr(lib, fn)(out.data_ptr(), phi.data_ptr(), f0.data_ptr(), _native.u64x3(d0),
                          _native.u64x3(d1), nc, nb, sett.bnd_array(), sett.nbnd,
                          _native.i32x3(sett.deg), sett.ext, _stream(f0))
    _native.check(fn, rc)
    return out


def pull(f0: torch.Tensor, phi: torch.Tensor, sett: Settings = Settings(), *, out=None) -> torch.Tensor:
    """Sample ``f₀`` at the 1-based voxel coordinates ``ϕ``; adjoint of ``push``.

    ``f₀ (d₀…, [C, [B]])``, ``ϕ (d₁…, 3, [B])`` -> ``f₁ (d₁…, [C, [B]])``."""
    return _pull_family("pp_pull", f0, phi, sett, (), out)


def pull_grad(f0: torch.Tensor, phi: torch.Tensor, sett: Settings = Settings(), *, out=None) -> torch.Tensor:
    """Spatial gradient of the interpolant at ``ϕ``: ``(d₁…, 3, [C, [B]])``; adjoint of ``push_grad``."""
    return _pull_family("pp_pull_grad", f0, phi, sett, (3,), out)


def pull_hess(f0: torch.Tensor, phi: torch.Tensor, sett: Settings = Settings(), *, out=None) -> torch.Tensor:
    """Hessian of the interpolant at ``ϕ``: ``(d₁…, 3, 3, [C, [B]])``."""
    return _pull_family("pp_pull_hess", f0, phi, sett, (3, 3), out)


def _push_family(fn: str, f1, phi, d0, sett: Settings, grad: bool, out=None, accumulate=False):
    if grad:
        assert 4 <= f1.dim() <= 6, "`∇f` must have between 4 & 6 dimensions"
        assert 4 <= phi.dim() <= 5, "`ϕ` must have 4 or 5 dimensions"
        assert L.jsize(phi, 4) == 3, "`ϕ` must have three channels"
        assert L.jsize(f1, 4) == 3, "`∇f` must have three components"
        assert L.jsize(phi, 5) == L.jsize(f1, 6), "`ϕ` & `∇f` must have the same batch size"
        assert tuple(f1.shape[:3]) == tuple(phi.shape[:3]), "`∇f` and `ϕ` must have the same volume dimensions"
        nc, nb, lead = L.jsize(f1, 5), L.jsize(f1, 6), 4
    else:
        assert 3 <= f1.dim() <= 5, "`f₁` must have between 3 & 5 dimensions"
        assert 4 <= phi.dim() <= 5, "`ϕ` must have 4 or 5 dimensions"
        assert L.jsize(phi, 4) == 3, "`ϕ` must have three channels"
        assert L.jsize(phi, 5) == L.jsize(f1, 5), "`ϕ` & `f₀` must have the same batch size"
        assert tuple(f1.shape[:3]) == tuple(phi.shape[:3]), "`f₁` and `ϕ` must have the same volume dimensions"
        nc, nb, lead = L.jsize(f1, 4), L.jsize(f1, 5), 3
    assert len(sett.bnd) == nc or len(sett.bnd) == 1
    _require_cuda(f1, phi)
    f1, phi = L.colmajor(f1), L.colmajor(phi)
    d0 = tuple(int(v) for v in d0)
    assert len(d0) == 3
    d1 = tuple(phi.shape[:3])
    shape = d0 + tuple(f1.shape[lead:])
    if out is None:
        out = L.empty(shape, device=f1.device)
        accumulate = False
    else:
        _require_cuda(out)
        assert tuple(out.shape) == shape and L.is_colmajor(out)
    lib = _native.lib()
    rc = getattr(lib, fn)(out.data_ptr(), phi.data_ptr(), f1.data_ptr(), _native.u64x3(d0),
                          _native.u64x3(d1), nc, nb, sett.bnd_array(), sett.nbnd,
                          _native.i32x3(sett.deg), sett.ext, int(bool(accumulate)), _stream(f1))
    _native.check(fn, rc)
    return out


def push(f1: torch.Tensor, phi: torch.Tensor, d0, sett: Settings = Settings(), *, out=None,
         accumulate: bool = False) -> torch.Tensor:
    """Scatter ``f₁`` through ``ϕ`` into a new ``d₀`` grid; adjoint of ``pull``.

    With ``out`` given and ``accumulate=True`` the values are added into ``out``."""
    return _push_family("pp_push", f1, phi, d0, sett, False, out, accumulate)


def push_grad(g1: torch.Tensor, phi: torch.Tensor, d0, sett: Settings = Settings(), *, out=None,
              accumulate: bool = False) -> torch.Tensor:
    """Adjoint of ``pull_grad``: ``∇f (d₁…, 3, [C, [B]])`` -> ``(d₀…, [C, [B]])``."""
    return _push_family("pp_push_grad", g1, phi, d0, sett, True, out, accumulate)


def push_count(f1: torch.Tensor, phi: torch.Tensor, d0, sett: Settings = Settings(), *, out=None, count=None,
               accumulate: bool = False):
    """``(push(f₁, ϕ), push(1, ϕ))`` in one pass: the pushed values and the
    weight every image voxel received from the same (finite, valid) samples
    (the reference's ``pushc``, artifacts/C/pushpull.cu:128-142)."""
    assert 3 <= f1.dim() <= 5, "`f₁` must have between 3 & 5 dimensions"
    assert 4 <= phi.dim() <= 5 and L.jsize(phi, 4) == 3
    assert L.jsize(phi, 5) == L.jsize(f1, 5) and tuple(f1.shape[:3]) == tuple(phi.shape[:3])
    nc, nb = L.jsize(f1, 4), L.jsize(f1, 5)
    assert len(sett.bnd) == nc or len(sett.bnd) == 1
    _require_cuda(f1, phi)
    f1, phi = L.colmajor(f1), L.colmajor(phi)
    d0 = tuple(int(v) for v in d0)
    shape = d0 + tuple(f1.shape[3:])
    if out is None or count is None:
        out, count, accumulate = L.empty(shape, device=f1.device), L.empty(shape, device=f1.device), False
    for t in (out, count):
        _require_cuda(t)
        assert tuple(t.shape) == shape and L.is_colmajor(t)
    lib = _native.lib()
    rc = lib.pp_push_count(out.data_ptr(), count.data_ptr(), phi.data_ptr(), f1.data_ptr(), _native.u64x3(d0),
                           _native.u64x3(tuple(phi.shape[:3])), nc, nb, sett.bnd_array(), sett.nbnd,
                           _native.i32x3(sett.deg), sett.ext, int(bool(accumulate)), _stream(f1))
    _native.check("pp_push_count", rc)
    return out, count


def adjust_affine(Aff) -> list:
    """1-based 3x4 (or 4x4) affine -> 0-based 3x4, column-major as 12 floats
    (src/pushpull_cpu.jl:357-362: the last column becomes the row sums minus 1,
    computed in Float32)."""
    A = torch.as_tensor(Aff, dtype=torch.float32).cpu()
    assert A.dim() == 2 and A.shape[1] == 4 and A.shape[0] in (3, 4)
    A = A[:3].clone()
    A[:, 3] = A.sum(dim=1) - 1.0
    return [float(v) for v in A.t().reshape(-1)]


def _affine_family(push: bool, x, Aff, d_other, sett: Settings, out=None, accumulate=False):
    assert 3 <= x.dim() <= 5, "input must have between 3 & 5 dimensions"
    assert len(sett.bnd) == L.jsize(x, 4) or len(sett.bnd) == 1
    _require_cuda(x)
    x = L.colmajor(x)
    nc, nb = L.jsize(x, 4), L.jsize(x, 5)
    d_other = tuple(int(v) for v in d_other)
    assert len(d_other) == 3
    d_in = tuple(x.shape[:3])
    d0, d1 = (d_other, d_in) if push else (d_in, d_other)
    shape = d_other + tuple(x.shape[3:])
    if out is None:
        out = L.empty(shape, device=x.device)
        accumulate = False
    else:
        _require_cuda(out)
        assert tuple(out.shape) == shape and L.is_colmajor(out)
    A = (C.c_float * 12)(*adjust_affine(Aff))
    lib = _native.lib()
    if push:
        rc = lib.pp_push_affine(out.data_ptr(), x.data_ptr(), A, _native.u64x3(d0), _native.u64x3(d1), nc, nb,
                                sett.bnd_array(), sett.nbnd, _native.i32x3(sett.deg), sett.ext,
                                int(bool(accumulate)), _stream(x))
        _native.check("pp_push_affine", rc)
    else:
        rc = lib.pp_pull_affine(out.data_ptr(), x.data_ptr(), A, _native.u64x3(d0), _native.u64x3(d1), nc, nb,
                                sett.bnd_array(), sett.nbnd, _native.i32x3(sett.deg), sett.ext, _stream(x))
        _native.check("pp_pull_affine", rc)
    return out


def affine_pull(f0: torch.Tensor, Aff, d1, sett: Settings = Settings(), *, out=None) -> torch.Tensor:
    """Sample ``f₀`` on a ``d₁`` grid mapped by the 1-based affine ``Aff`` (3x4 or
    4x4): ``f₁[i] = f₀(Aff * i)`` (src/pushpull_cpu.jl:268-307)."""
    return _affine_family(False, f0, Aff, d1, sett, out)


def affine_push(f1: torch.Tensor, Aff, d0, sett: Settings = Settings(), *, out=None,
                accumulate: bool = False) -> torch.Tensor:
    """Adjoint of ``affine_pull``: scatter ``f₁`` into a ``d₀`` grid
    (src/pushpull_cpu.jl:310-349)."""
    return _affine_family(True, f1, Aff, d0, sett, out, accumulate)


def id(v: torch.Tensor = None, *, affine=None, dim=None, device=None) -> torch.Tensor:  # noqa: A001
    """1-based identity deformation ``(d…, 3)``, optionally affine (src/pushpull_general.jl:81-99)."""
    if dim is None:
        dim = tuple(v.shape[:3])
    if device is None:
        device = v.device if v is not None else "cuda"
    x = torch.arange(1, dim[0] + 1, dtype=torch.float32, device=device).view(-1, 1, 1)
    y = torch.arange(1, dim[1] + 1, dtype=torch.float32, device=device).view(1, -1, 1)
    z = torch.arange(1, dim[2] + 1, dtype=torch.float32, device=device).view(1, 1, -1)
    phi = L.empty(tuple(dim) + (3,), device=device)
    if affine is None:
        phi[..., 0] = x
        phi[..., 1] = y
        phi[..., 2] = z
    else:
        A = [[float(a) for a in row] for row in affine]
        for k in range(3):
            phi[..., k] = (A[k][0] * x.double() + A[k][1] * y.double() + A[k][2] * z.double()
                           + A[k][3]).float()
    return phi


def _dot_family(fn: str, f0, phi, up, sett: Settings, up_comps: int):
    assert 3 <= f0.dim() <= 5, "`f₀` must have between 3 & 5 dimensions"
    assert 4 <= phi.dim() <= 5, "`ϕ` must have 4 or 5 dimensions"
    assert L.jsize(phi, 4) == 3, "`ϕ` must have three channels"
    assert L.jsize(phi, 5) == L.jsize(f0, 5), "`ϕ` & `f₀` must have the same batch size"
    nc, nb = L.jsize(f0, 4), L.jsize(f0, 5)
    assert len(sett.bnd) == nc or len(sett.bnd) == 1
    d1 = tuple(phi.shape[:3])
    want = d1 + ((3,) if up_comps == 3 else ()) + (nc, nb)
    assert up.numel() == int(torch.tensor(want).prod()), "upstream does not match the sample grid"
    _require_cuda(f0, phi, up)
    f0, phi, up = L.colmajor(f0), L.colmajor(phi), L.colmajor(up)
    out = L.empty(tuple(phi.shape), device=f0.device)
    lib = _native.lib()
    rc = getattr(lib, fn)(out.data_ptr(), phi.data_ptr(), f0.data_ptr(), up.data_ptr(),
                          _native.u64x3(f0.shape[:3]), _native.u64x3(d1), nc, nb, sett.bnd_array(), sett.nbnd,
                          _native.i32x3(sett.deg), sett.ext, _stream(f0))
    _native.check(fn, rc)
    return out


def pull_grad_dot(f0: torch.Tensor, phi: torch.Tensor, up: torch.Tensor, sett: Settings = Settings()) -> torch.Tensor:
    """``Σ_c up_c · ∇pull(f₀_c, ϕ)`` with the shape of ``ϕ``: the ϕ-cotangent of ``pull``
    (src/pushpull_pb.jl:11-18) without the ``(d₁…, 3, C, B)`` temporary."""
    return _dot_family("pp_pull_grad_dot", f0, phi, up, sett, 1)


def pull_hess_dot(f0: torch.Tensor, phi: torch.Tensor, up: torch.Tensor, sett: Settings = Settings()) -> torch.Tensor:
    """``Σ_c H_c · up_c`` with the shape of ``ϕ``: the ϕ-cotangent of ``pull_grad``
    (src/pushpull_pb.jl:26-35); ``up`` has the shape of a ``pull_grad`` output."""
    return _dot_family("pp_pull_hess_dot", f0, phi, up, sett, 3)


def fused_step(f0: torch.Tensor, phi: torch.Tensor, g: torch.Tensor, sett: Settings = Settings(), *,
               df_out=None, accumulate: bool = False):
    """Loss ``Σ (pull(f₀, ϕ) - g)²`` and its gradients in one pass.

    Returns ``(loss, df, dphi)``: ``loss`` a 0-d float64 CUDA tensor, ``df`` with the
    shape of ``f₀`` (= push(2r)), ``dphi`` with the shape of ``ϕ`` (= Σ_c 2r_c ∇pull_c)."""
    assert 3 <= f0.dim() <= 5 and 4 <= phi.dim() <= 5 and L.jsize(phi, 4) == 3
    assert L.jsize(phi, 5) == L.jsize(f0, 5), "`ϕ` & `f₀` must have the same batch size"
    nc, nb = L.jsize(f0, 4), L.jsize(f0, 5)
    assert len(sett.bnd) == nc or len(sett.bnd) == 1
    d1 = tuple(phi.shape[:3])
    assert tuple(g.shape[:3]) == d1 and g.numel() == int(torch.tensor(d1).prod()) * nc * nb, \
        "`g` must have the shape of pull(f₀, ϕ)"
    _require_cuda(f0, phi, g)
    f0, phi, g = L.colmajor(f0), L.colmajor(phi), L.colmajor(g)
    if df_out is None:
        df = L.empty(tuple(f0.shape), device=f0.device)
        accumulate = False
    else:
        _require_cuda(df_out)
        assert tuple(df_out.shape) == tuple(f0.shape) and L.is_colmajor(df_out)
        df = df_out
    dphi = L.empty(tuple(phi.shape), device=f0.device)
    loss = torch.empty((), dtype=torch.float64, device=f0.device)
    lib = _native.lib()
    rc = lib.pp_fused_step(loss.data_ptr(), df.data_ptr(), dphi.data_ptr(), f0.data_ptr(), phi.data_ptr(),
                           g.data_ptr(), _native.u64x3(f0.shape[:3]), _native.u64x3(d1), nc, nb,
                           sett.bnd_array(), sett.nbnd, _native.i32x3(sett.deg), sett.ext, int(bool(accumulate)),
                           _stream(f0))
    _native.check("pp_fused_step", rc)
    return loss, df, dphi
