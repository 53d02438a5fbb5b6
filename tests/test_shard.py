"""Data-parallel sharding (pushpull_gb300.shard) on CPU ranks: two gloo
processes split the sample grid into z-slabs; the gathered pull equals the
single-process result exactly, the all-reduced push equals it to rounding.
The slab compute is the FP64 oracle here (the partition and the collective are
what is under test; a GPU rank runs the same code with the CUDA ops)."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _oracle_ops():
    import __graft_entry__ as entry
    pkg = entry.package()
    from oracle import oracle as O
    L = pkg.layout
    so = O.Sett.make(3, 1, 1)

    def pull_op(f0, phi, sett):
        return L.from_numpy(O.pull(L.to_numpy(f0), L.to_numpy(phi), so), device="cpu")

    def push_op(f1, phi, d0, sett):
        return L.from_numpy(O.push(L.to_numpy(f1), L.to_numpy(phi), d0, so), device="cpu")
    return pkg, O, so, pull_op, push_op


def _inputs(O):
    rng = np.random.default_rng(7)
    d0, d1 = (14, 12, 9), (13, 11, 7)
    f0 = np.asfortranarray(rng.standard_normal(d0).astype(np.float32))
    phi = O.identity(d1).astype(np.float64)
    phi = np.asfortranarray((phi + rng.standard_normal(phi.shape)).astype(np.float32))
    f1 = np.asfortranarray(rng.standard_normal(d1).astype(np.float32))
    return d0, f0, phi, f1


def _rank_main(rank, world, port, outdir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        pkg, O, so, pull_op, push_op = _oracle_ops()
        from pushpull_gb300 import shard
        L = pkg.layout
        d0, f0, phi, f1 = _inputs(O)
        tf0, tphi, tf1 = (L.from_numpy(a, device="cpu") for a in (f0, phi, f1))
        got1 = shard.pull_sharded(pull_op, tf0, tphi, None)
        got0 = shard.push_sharded(push_op, tf1, tphi, d0, None)
        local, (z0, z1) = shard.pull_sharded(pull_op, tf0, tphi, None, gather=False)
        np.savez(os.path.join(outdir, f"rank{rank}.npz"), pull=L.to_numpy(got1), push=L.to_numpy(got0),
                 local=L.to_numpy(local), z=np.array([z0, z1]))
    finally:
        dist.destroy_process_group()


def test_slab_and_split_items():
    from importlib import import_module
    import __graft_entry__ as entry
    entry.package()
    shard = import_module("pushpull_gb300.shard")
    for n in (1, 2, 7, 192):
        for w in (1, 2, 3, 8):
            parts = [shard.slab(n, r, w) for r in range(w)]
            assert parts[0][0] == 0 and parts[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(parts, parts[1:]))
            assert max(b - a for a, b in parts) - min(b - a for a, b in parts) <= 1
    owner = shard.split_items([5, 1, 9, 3, 3, 8], 2)
    assert sorted(i for o in owner for i in o) == list(range(6))
    loads = [sum([5, 1, 9, 3, 3, 8][i] for i in o) for o in owner]
    assert abs(loads[0] - loads[1]) <= 2


def test_two_gloo_ranks_match_single_process(tmp_path):
    world = 2
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, str(tmp_path))) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
    for p in procs:
        if p.is_alive():
            p.kill()
            pytest.fail("gloo rank hung")
        assert p.exitcode == 0
    pkg, O, so, _, _ = _oracle_ops()
    d0, f0, phi, f1 = _inputs(O)
    ref1 = O.pull(f0, phi, so)
    ref0 = O.push(f1, phi, d0, so)
    slabs = []
    for r in range(world):
        z = np.load(tmp_path / f"rank{r}.npz")
        assert np.array_equal(z["pull"], ref1.astype(z["pull"].dtype), equal_nan=True)
        assert np.allclose(z["push"], ref0, rtol=1e-12, atol=1e-12 * np.abs(ref0).max())
        z0, z1 = z["z"]
        slabs.append((z0, z1))
        assert np.array_equal(z["local"], ref1[:, :, z0:z1].astype(z["local"].dtype), equal_nan=True)
    assert slabs[0][0] == 0 and slabs[-1][1] == phi.shape[2] and slabs[0][1] == slabs[1][0]
