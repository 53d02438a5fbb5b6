"""Seeded synthetic volumes and deformations for the benchmark workloads.

No public dataset is involved; these stand in for the workloads with the stated
shapes and value distributions:

* images: i.i.d. U(0,1), Gaussian-smoothed (FWHM in voxels, sigma = FWHM/2.3548,
  periodic boundary);
* deformations: 1-based identity plus a displacement made of one seeded N(0,1)
  field per component, smoothed, then scaled so that max|u| equals the stated
  amplitude (optionally composed with a global contraction about the centre).

Everything is Float32 in the reference's column-major layout (numpy Fortran order).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

FWHM_TO_SIGMA = 1.0 / 2.3548


def _smooth(a: np.ndarray, fwhm: float) -> np.ndarray:
    from scipy.ndimage import gaussian_filter
    return gaussian_filter(a, sigma=fwhm * FWHM_TO_SIGMA, mode="wrap")


def image(d, seed: int, fwhm: float = 3.0, channels: int = 1) -> np.ndarray:
    rng = np.random.default_rng(seed)
    vols = [_smooth(rng.random(tuple(d)).astype(np.float32), fwhm) for _ in range(channels)]
    out = np.stack(vols, axis=-1) if channels > 1 else vols[0]
    return np.asfortranarray(out.astype(np.float32))


def identity(d) -> np.ndarray:
    x = np.arange(1, d[0] + 1, dtype=np.float32)[:, None, None]
    y = np.arange(1, d[1] + 1, dtype=np.float32)[None, :, None]
    z = np.arange(1, d[2] + 1, dtype=np.float32)[None, None, :]
    phi = np.empty(tuple(d) + (3,), dtype=np.float32, order="F")
    phi[..., 0], phi[..., 1], phi[..., 2] = x, y, z
    return phi


def deformation(d, seed: int, fwhm: float, amplitude: float, contraction: float = 1.0,
                d_src=None) -> np.ndarray:
    """identity (optionally scaled by ``contraction`` about the centre of ``d_src``)
    plus a smoothed random field with max|u| = amplitude."""
    rng = np.random.default_rng(seed)
    d = tuple(int(v) for v in d)
    d_src = tuple(int(v) for v in (d_src or d))
    phi = identity(d).astype(np.float64)
    for k in range(3):
        # map the sample grid onto the source grid, then contract about its centre
        scale = (d_src[k] - 1) / max(d[k] - 1, 1)
        x = 1.0 + (phi[..., k] - 1.0) * scale
        c = 0.5 * (d_src[k] + 1)
        phi[..., k] = c + contraction * (x - c)
    u = np.stack([_smooth(rng.standard_normal(d).astype(np.float32), fwhm) for _ in range(3)], axis=-1)
    m = float(np.abs(u).max())
    if m > 0:
        u *= amplitude / m
    return np.asfortranarray((phi + u).astype(np.float32))


@dataclass
class Workload:
    name: str
    f0: np.ndarray          # (d0..., [C])
    phi: np.ndarray         # (d1..., 3)
    deg: tuple
    bnd: object
    ext: int
    extra: dict


def config1(seed: int = 1) -> Workload:
    """64^3, degree 1, circulant, ext = 0; FWHM-8 field scaled to +-2 vox."""
    d = (64, 64, 64)
    return Workload("pull+push 64^3 trilinear circulant ext=0", image(d, seed), deformation(d, seed + 1, 8.0, 2.0),
                    (1, 1, 1), 0, 0, {})


def config2(seed: int = 2) -> Workload:
    """192^3, degree 3, DCT-II, ext = 1; FWHM-12 field scaled to +-5 vox; 1 channel."""
    d = (192, 192, 192)
    return Workload("pull+push 192^3 cubic DCT2 ext=1", image(d, seed), deformation(d, seed + 1, 12.0, 5.0),
                    (3, 3, 3), 1, 1, {})


def config3(seed: int = 3) -> Workload:
    """160x192x160, degree 2, bounds (circulant, DCT-II, DST-II); target g = pull(f, phi2)."""
    d = (160, 192, 160)
    w = Workload("fused step 160x192x160 quadratic mixed bounds", image(d, seed),
                 deformation(d, seed + 1, 12.0, 3.0), (2, 2, 2), (0, 1, 2), 1, {})
    w.extra["phi2"] = deformation(d, seed + 2, 12.0, 3.0)
    return w


def config5(seed: int = 5) -> Workload:
    """256^3 x 3 channels, degree 3, DCT-II; 0.25x contraction about the centre + field +-3 vox."""
    d = (256, 256, 256)
    return Workload("push 256^3x3 cubic DCT2 contraction", image(d, seed, channels=3),
                    deformation(d, seed + 1, 12.0, 3.0, contraction=0.25), (3, 3, 3), 1, 1, {})


def affine_map(d, seed: int = 6) -> np.ndarray:
    """1-based 4x4 affine of a d grid onto itself: rotations of up to 10 degrees
    about each axis and scalings in [0.9, 1.1] about the centre, plus a shift of
    up to 3 voxels (a rigid-plus-zoom registration update)."""
    rng = np.random.default_rng(seed)
    th = rng.uniform(-np.pi / 18, np.pi / 18, 3)
    c, s = np.cos(th), np.sin(th)
    R = (np.array([[1, 0, 0], [0, c[0], -s[0]], [0, s[0], c[0]]])
         @ np.array([[c[1], 0, s[1]], [0, 1, 0], [-s[1], 0, c[1]]])
         @ np.array([[c[2], -s[2], 0], [s[2], c[2], 0], [0, 0, 1]]))
    M = R @ np.diag(rng.uniform(0.9, 1.1, 3))
    ctr = 0.5 * (np.array(d, dtype=np.float64) + 1)
    A = np.eye(4, dtype=np.float32)
    A[:3, :3] = M
    A[:3, 3] = ctr - M @ ctr + rng.uniform(-3, 3, 3)
    return A


def batched_pairs(seed: int = 4, npairs: int = 32, levels: int = 3):
    """Uneven batch: sizes uniform in [64,256]x[64,256]x[64,192], 1-3 channels,
    degree from {1,2,3}; each pair with a pyramid of ``levels`` (each level halved)."""
    rng = np.random.default_rng(seed)
    items = []
    for p in range(npairs):
        d = (int(rng.integers(64, 257)), int(rng.integers(64, 257)), int(rng.integers(64, 193)))
        c = int(rng.integers(1, 4))
        deg = int(rng.choice([1, 2, 3]))
        for lev in range(levels):
            dl = tuple(max(1, (v + (1 << lev) - 1) >> lev) for v in d)
            items.append(dict(pair=p, level=lev, d=dl, channels=c, deg=deg, seed=seed * 1000 + p * 10 + lev))
    return items


# ---- device-side generation (the batched workload has ~100 volumes) ---------
def _smooth_gpu(vol, fwhm: float):
    """Periodic Gaussian smoothing of a (X, Y, Z) float32 CUDA tensor by FFT."""
    import torch
    sigma = fwhm * FWHM_TO_SIGMA
    F = torch.fft.rfftn(vol.double())
    for ax, n in enumerate(vol.shape):
        k = torch.fft.rfftfreq(n, device=vol.device) if ax == vol.dim() - 1 else torch.fft.fftfreq(n, device=vol.device)
        h = torch.exp(-2.0 * (torch.pi * sigma * k.double()) ** 2)
        shape = [1] * vol.dim()
        shape[ax] = -1
        F = F * h.view(shape)
    return torch.fft.irfftn(F, s=vol.shape).float()


def image_gpu(d, seed: int, fwhm: float = 3.0, channels: int = 1, device="cuda"):
    """Column-major (d..., [C]) image: U(0,1) i.i.d. smoothed with FWHM ``fwhm``."""
    import torch
    from . import layout as L
    g = torch.Generator(device=device).manual_seed(seed)
    out = L.empty(tuple(d) + ((channels,) if channels > 1 else ()), device=device)
    for c in range(channels):
        v = torch.rand(tuple(d), generator=g, device=device)
        sm = _smooth_gpu(v, fwhm)
        if channels > 1:
            out[..., c] = sm
        else:
            out.copy_(sm)
    return out


def deformation_gpu(d, seed: int, fwhm: float, amplitude: float, contraction: float = 1.0, device="cuda"):
    """Column-major (d..., 3): 1-based identity (optionally scaled by
    ``contraction`` about the volume centre) + smoothed N(0,1) field, max|u| = amplitude."""
    import torch
    from . import layout as L
    g = torch.Generator(device=device).manual_seed(seed)
    phi = L.empty(tuple(d) + (3,), device=device)
    u = torch.stack([_smooth_gpu(torch.randn(tuple(d), generator=g, device=device), fwhm) for _ in range(3)], -1)
    u *= amplitude / u.abs().max()
    ax = [0.5 * (n + 1) + contraction * (torch.arange(1, n + 1, dtype=torch.float32, device=device) - 0.5 * (n + 1))
          for n in d]
    phi[..., 0] = ax[0].view(-1, 1, 1) + u[..., 0]
    phi[..., 1] = ax[1].view(1, -1, 1) + u[..., 1]
    phi[..., 2] = ax[2].view(1, 1, -1) + u[..., 2]
    return phi
