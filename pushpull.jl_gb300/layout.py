"""Julia (column-major) layout for torch tensors.

The library works on the reference's memory layout: a volume of Julia shape
``(d1, d2, d3, C, B)`` is stored with the first index fastest.  In torch that
is a tensor of that shape with strides ``(1, d1, d1*d2, ...)`` -- the transpose
view of a contiguous ``(B, C, d3, d2, d1)`` tensor -- so the shapes and the
``size(a, k)`` arithmetic read exactly as in the reference.
"""
from __future__ import annotations

import numpy as np
import torch


def colmajor_strides(shape) -> tuple:
    out, s = [], 1
    for d in shape:
        out.append(s)
        s *= int(d)
    return tuple(out)


def is_colmajor(t: torch.Tensor) -> bool:
    want = colmajor_strides(t.shape)
    return all(d == 1 or st == w for d, st, w in zip(t.shape, t.stride(), want))


def _rev(n: int) -> tuple:
    return tuple(range(n - 1, -1, -1))


def empty(shape, device="cuda", dtype=torch.float32) -> torch.Tensor:
    shape = tuple(int(s) for s in shape)
    return torch.empty(shape[::-1], device=device, dtype=dtype).permute(*_rev(len(shape)))


def zeros(shape, device="cuda", dtype=torch.float32) -> torch.Tensor:
    shape = tuple(int(s) for s in shape)
    return torch.zeros(shape[::-1], device=device, dtype=dtype).permute(*_rev(len(shape)))


def full(shape, value, device="cuda", dtype=torch.float32) -> torch.Tensor:
    shape = tuple(int(s) for s in shape)
    return torch.full(shape[::-1], value, device=device, dtype=dtype).permute(*_rev(len(shape)))


def colmajor(t: torch.Tensor) -> torch.Tensor:
    """``t`` itself if already column-major, else a column-major copy."""
    if is_colmajor(t):
        return t
    r = _rev(t.dim())
    return t.permute(*r).contiguous().permute(*r)


def from_numpy(a: np.ndarray, device="cuda") -> torch.Tensor:
    """Fortran-ordered numpy array -> column-major torch tensor of the same shape."""
    a = np.asfortranarray(a)
    flat = torch.from_numpy(np.ascontiguousarray(a.ravel(order="F")))
    t = flat.reshape(a.shape[::-1]).permute(*_rev(a.ndim))
    return t.to(device) if device is not None else t


def to_numpy(t: torch.Tensor) -> np.ndarray:
    """Column-major torch tensor -> Fortran-ordered numpy array of the same shape."""
    r = _rev(t.dim())
    c = t.detach().permute(*r).contiguous().cpu().numpy()   # C order, reversed shape
    return c.transpose(*r)


def reshape(t: torch.Tensor, shape) -> torch.Tensor:
    """Julia ``reshape`` (column-major element order) of a column-major tensor."""
    t = colmajor(t)
    r = _rev(t.dim())
    flat = t.permute(*r).reshape(-1)
    shape = tuple(int(s) for s in shape)
    return flat.reshape(shape[::-1]).permute(*_rev(len(shape)))


def flat(t: torch.Tensor) -> torch.Tensor:
    """The elements of a column-major tensor in column-major order, as a 1-D view
    (a copy only if ``t`` is not column-major)."""
    t = colmajor(t)
    return t.permute(*_rev(t.dim())).reshape(-1)


def unflat(v: torch.Tensor, shape) -> torch.Tensor:
    """Inverse of ``flat``: a 1-D tensor viewed as a column-major tensor of ``shape``."""
    shape = tuple(int(s) for s in shape)
    return v.reshape(shape[::-1]).permute(*_rev(len(shape)))


def jsize(t, k: int) -> int:
    """Julia ``size(t, k)`` (1-based; 1 beyond ndims)."""
    return int(t.shape[k - 1]) if k <= t.dim() else 1
