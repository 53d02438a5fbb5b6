"""Data-parallel sharding of the pull / push path over ranks (one GPU each).

The path partitions without a halo exchange:

* pull family (pull, pull_grad, pull_hess): the sample grid is split into
  z-slabs; rank r evaluates its slab of the deformation against the whole
  image (the image region a slab touches is unknown until its deformation has
  been read, so every rank holds the image) and the slabs are gathered.
* push family (push, push_grad): the samples are split the same way; each rank
  scatters its slab into a private image of the full size and the private
  images are summed with one all-reduce (the only collective on the path).
* uneven batches of independent volumes split by volume with no exchange
  (``split_items``).

The reference has no multi-device path (ext/pushpull_gpu.jl launches on the
current device only); this module is the data-parallel layer a multi-GPU user
of the library calls.  ``op`` is any function with the signature of the
package's pull / push functions, so the partition and reduction logic is the
same whatever computes the slabs.
"""
from __future__ import annotations

import torch
import torch.distributed as dist

from . import layout as L


def slab(n: int, rank: int, world: int) -> tuple:
    """Balanced split of range(n) into `world` contiguous slabs: rank's (z0, z1)."""
    base, extra = divmod(n, world)
    z0 = rank * base + min(rank, extra)
    return z0, z0 + base + (1 if rank < extra else 0)


def _world(group):
    if dist.is_available() and dist.is_initialized():
        return dist.get_rank(group), dist.get_world_size(group)
    return 0, 1


def _zslice(t: torch.Tensor, z0: int, z1: int) -> torch.Tensor:
    return L.colmajor(t[:, :, z0:z1])


def pull_sharded(op, f0: torch.Tensor, phi: torch.Tensor, sett, group=None, gather: bool = True):
    """``op(f0, phi_slab, sett)`` on this rank's z-slab of the sample grid; with
    ``gather`` the full result on every rank, else (local slab, (z0, z1))."""
    rank, world = _world(group)
    nz = phi.shape[2]
    z0, z1 = slab(nz, rank, world)
    local = op(f0, _zslice(phi, z0, z1), sett)
    if not gather or world == 1:
        return local if world == 1 else (local, (z0, z1))
    # gather compact slabs (padded to the largest) and place them along z
    zmax = max(slab(nz, r, world)[1] - slab(nz, r, world)[0] for r in range(world))
    shape = list(local.shape)
    shape[2] = zmax
    padded = L.zeros(tuple(shape), device=local.device, dtype=local.dtype)
    padded[:, :, : z1 - z0] = local
    flat = L.flat(padded)
    parts = [torch.empty_like(flat) for _ in range(world)]
    dist.all_gather(parts, flat, group=group)
    out_shape = list(local.shape)
    out_shape[2] = nz
    out = L.empty(tuple(out_shape), device=local.device, dtype=local.dtype)
    for r, part in enumerate(parts):
        r0, r1 = slab(nz, r, world)
        out[:, :, r0:r1] = L.unflat(part, tuple(shape))[:, :, : r1 - r0]
    return out


def push_sharded(op, f1: torch.Tensor, phi: torch.Tensor, d0, sett, group=None):
    """Sum over ranks of ``op(f1_slab, phi_slab, d0, sett)``: the full push on every rank."""
    rank, world = _world(group)
    nz = phi.shape[2]
    z0, z1 = slab(nz, rank, world)
    local = op(_zslice(f1, z0, z1), _zslice(phi, z0, z1), d0, sett)
    if world > 1:
        flat = L.flat(local)
        dist.all_reduce(flat, op=dist.ReduceOp.SUM, group=group)
        local = L.unflat(flat, tuple(local.shape))
    return local


def split_items(costs, world: int) -> list:
    """Assign independent volumes (cost = voxels x channels) to ranks, largest
    first onto the least-loaded rank; returns one index list per rank."""
    load = [0] * world
    owner = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda k: -costs[k]):
        r = min(range(world), key=lambda q: load[q])
        owner[r].append(i)
        load[r] += costs[i]
    return [sorted(o) for o in owner]
