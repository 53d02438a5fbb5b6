"""Benchmark: pull + push throughput at 192^3, cubic B-spline, DCT-II bounds, ext = 1.

One step = one pull of a 192^3 Float32 image through a 192^3 deformation
(identity + FWHM-12 smoothed random field scaled to +-5 voxels) followed by one
push of the pulled values back through the same deformation.  ``value`` is
Gvox/s (sample voxels x channels per second, whole job) from CUDA events around
each step with inputs resident in HBM and L2 flushed before each step; ``e2e``
is the same step through the reference-facing host-pointer ABI (the ``pull`` /
``push`` symbols of artifacts/C/pushpull.h) with pinned host buffers.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

``--impl reference`` times the reference CPU implementation of the path on the
host cores instead (compiled from the reference sources where possible, else the
CPU port of it), on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "pull+push Gvox/s & HBM GB/s @192³ cubic; fused fwd+adjoint vs plain GPU"
L2_FLUSH_BYTES = 256 << 20
# GPU cycles of a spin kernel queued after each L2 flush and before the start
# event: the host enqueues the timed calls meanwhile, so the events bracket
# device work only (host-side argument handling is timed by the e2e leg)
HOST_AHEAD_CYCLES = 400_000


def _flush(buf):
    import torch
    buf.fill_(1.0)
    torch.cuda._sleep(HOST_AHEAD_CYCLES)


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _errors(got, ref, floor=1e-3):
    """FP64-oracle error of a result: norm-wise max|a-b| / max|b| and elementwise
    max |a-b| / |b| over entries with |b| > floor * max|b| (NaN entries must agree)."""
    a = np.asarray(got, np.float64).ravel(order="F")
    b = np.asarray(ref, np.float64).ravel(order="F")
    nan_ok = bool((np.isnan(a) == np.isnan(b)).all())
    m = ~np.isnan(b)
    a, b = a[m], b[m]
    if b.size == 0:
        return {"norm": 0.0, "elem": 0.0, "elem_floor": floor, "nan_masks_equal": nan_ok}
    mx = float(np.abs(b).max())
    big = np.abs(b) > floor * mx
    norm = float(np.abs(a - b).max() / mx) if mx > 0 else float(np.abs(a).max())
    elem = float((np.abs(a[big] - b[big]) / np.abs(b[big])).max()) if big.any() else 0.0
    return {"norm": norm, "elem": elem, "elem_floor": floor, "nan_masks_equal": nan_ok}


def _oracle_threads():
    return max(1, min(32, os.cpu_count() or 1))


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch of each kernel on this
# workload, from one ncu capture each (profiles/k_pull_ws_192cubic.md, k_push_tiled_192cubic.md,
# k_pull_ws_affine_192cubic.md, k_push_tiled_affine_192cubic.md)
TRAFFIC = {"pull": 125_749_248, "push": 152_941_824, "affine_pull": 28_637_184, "affine_push": 56_648_448}


class Clocks:
    """Samples nvidia-smi every 200 ms while the timed region runs."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid):
        self.uuid, self.proc, self.path = uuid, None, None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            cmd = ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "200"]
            if self.uuid:
                cmd += ["-i", self.uuid]
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(cmd, stdout=self.fh, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not self.path:
            return None
        rows = []
        with open(self.path) as fh:
            for line in fh:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 8:
                    continue
                try:
                    rows.append((float(parts[0]), float(parts[1]), float(parts[2]), parts[3:]))
                except ValueError:
                    continue
        os.unlink(self.path)
        if not rows:
            return None
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[3][1:]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "power_w_max": max(r[2] for r in rows), "samples": len(rows), "reasons": sorted(reasons)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _workload(args):
    from pushpull_gb300 import workloads
    w = workloads.config2(seed=args.seed)
    return w


def cpu_baseline(w, seconds=8.0, kind=None):
    from oracle.cpu_bench import PullPushCPU
    h = PullPushCPU(w.f0, w.phi, w.deg, w.bnd, w.ext, kind=kind)
    h.step()                                   # warm-up
    times = []
    t_end = time.perf_counter() + seconds
    while time.perf_counter() < t_end or len(times) < 2:
        times.append(h.step())
    n1 = h.n1
    h.close()
    sec = statistics.mean(times)
    return {"value": n1 / sec / 1e9, "unit": "Gvox/s", "cores": h.threads, "kind": h.kind,
            "sample": f"full workload: pull + push of all {n1} voxels per rep, {len(times)} reps "
                      f"({sum(times):.1f} s), {h.threads} threads over contiguous voxel slabs"}, sec


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    w = _workload(args)
    from oracle.cpu_bench import PullPushCPU
    h = PullPushCPU(w.f0, w.phi, w.deg, w.bnd, w.ext)
    for _ in range(args.warmup):
        h.step()
    times = [h.step() for _ in range(args.steps)]
    h.close()
    sec = statistics.mean(times)
    value = h.n1 / sec / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Gvox/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": _config(w, args),
            "cpu_baseline": {"value": value, "unit": "Gvox/s", "cores": h.threads, "kind": h.kind,
                             "sample": f"pull + push of all {h.n1} voxels per step, {h.threads} threads"},
            "e2e": {"value": value, "unit": "Gvox/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def _config(w, args):
    return {"workload": "pull then push, 192x192x192 Float32, 1 channel, degree 3 (cubic) all dims, "
                        "DCT-II bounds, extrapolate=true, phi = identity + FWHM-12 smoothed N(0,1) field "
                        "scaled to +-5 vox",
            "d": list(w.f0.shape[:3]), "deg": list(w.deg), "bnd": w.bnd, "ext": w.ext, "channels": 1,
            "seed": args.seed,
            "l2": f"flushed before every step by a {L2_FLUSH_BYTES >> 20} MiB write outside the step's events",
            "timing": f"CUDA events on the launch stream; a {HOST_AHEAD_CYCLES}-cycle GPU spin before each start "
                      "event lets the host enqueue the step first, so the events bracket device work"}


def run_gpu(args):
    import torch
    import torch.distributed as dist

    import __graft_entry__ as entry
    pkg = entry.package()
    L = pkg.layout
    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=dev)

    w = _workload(args)
    d0 = tuple(w.f0.shape[:3])
    d1 = tuple(w.phi.shape[:3])
    n0, n1 = int(np.prod(d0)), int(np.prod(d1))
    nc = 1
    s = pkg.Settings(w.deg, w.bnd, w.ext)
    f0 = L.from_numpy(w.f0, dev)
    phi = L.from_numpy(w.phi, dev)
    f1 = L.empty(d1, device=dev)
    acc = L.empty(d0, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def step(evs=None):
        _flush(flush)
        if evs:
            evs[0].record()
        pkg.pull(f0, phi, s, out=f1)
        if evs:
            evs[1].record()
        pkg.push(f1, phi, d0, s, out=acc, accumulate=False)
        if evs:
            evs[2].record()

    for _ in range(max(args.warmup, 3)):
        step()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    uuid = None
    try:
        uuid = str(torch.cuda.get_device_properties(dev).uuid)
        uuid = uuid if uuid.startswith("GPU-") else "GPU-" + uuid
    except Exception:
        pass
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with Clocks(uuid if rank == 0 else None) as clk:
        t0 = time.perf_counter()
        for i in range(args.steps):
            step(evs[i])
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    if ws > 1:
        dist.barrier()
    # pull_grad of the same image and deformation (outside the timed pull+push step)
    g1 = L.empty(d1 + (3,), device=dev)
    pg_ms = []
    for i in range(max(args.steps, 5) + 3):
        _flush(flush)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        pkg.pull_grad(f0, phi, s, out=g1)
        e1.record()
        torch.cuda.synchronize()
        if i >= 3:
            pg_ms.append(e0.elapsed_time(e1))
    # push_grad of that gradient field back through the same deformation
    accg = L.empty(d0, device=dev)
    pushg_ms = _timeit(lambda: pkg.push_grad(g1, phi, d0, s, out=accg, accumulate=False), max(args.steps, 5), flush)
    del g1, accg
    # affine pull and push of the same image (positions A (i, j, k, 1) computed
    # in the kernels in place of a deformation), outside the timed step
    from pushpull_gb300 import workloads as W
    Aff = W.affine_map(d0, seed=args.seed + 4)
    fa = L.empty(d1, device=dev)
    aa = L.empty(d0, device=dev)
    reps = max(args.steps, 5)
    aff_pull_ms = _timeit(lambda: pkg.affine_pull(f0, Aff, d1, s, out=fa), reps, flush)
    aff_push_ms = _timeit(lambda: pkg.affine_push(fa, Aff, d0, s, out=aa), reps, flush)
    # FP64 error of the benchmarked pull and push (outside every timed region):
    # f1 and acc hold the last timed step's outputs
    accuracy = None
    if not args.no_accuracy:
        from oracle import oracle as O
        so = O.Sett.make(w.deg, w.bnd, w.ext)
        th = _oracle_threads()
        f1n = L.to_numpy(f1)
        fan = L.to_numpy(fa)
        accuracy = {"pull": _errors(f1n, O.pull(w.f0, w.phi, so, threads=th)),
                    "push": _errors(L.to_numpy(acc), O.push(f1n, w.phi, d0, so, threads=th)),
                    "affine_pull": _errors(fan, O.pull_affine(w.f0, Aff, d1, so)),
                    "affine_push": _errors(L.to_numpy(aa), O.push_affine(fan, Aff, d0, so)),
                    "reference": "FP64 oracle (oracle/pp_oracle.c) on the same inputs, whole volume"}
    pull_ms = [e[0].elapsed_time(e[1]) for e in evs]
    push_ms = [e[1].elapsed_time(e[2]) for e in evs]
    step_ms = statistics.mean(a + b for a, b in zip(pull_ms, push_ms))
    if ws > 1:
        t = torch.tensor([step_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        step_ms = float(t.item())
    value = ws * n1 * nc / (step_ms * 1e-3) / 1e9

    # ---- end to end through the reference-facing host ABI (pinned host buffers)
    e2e = None
    if not args.no_e2e:
        import ctypes as C
        lib = pkg.native_library()
        hf0 = torch.from_numpy(np.ascontiguousarray(w.f0.ravel(order="F"))).pin_memory()
        hphi = torch.from_numpy(np.ascontiguousarray(w.phi.ravel(order="F"))).pin_memory()
        hf1 = torch.empty(n1, dtype=torch.float32).pin_memory()
        hacc = torch.empty(n0, dtype=torch.float32).pin_memory()
        cd0 = (C.c_ulonglong * 3)(*d0)
        cb = (C.c_int * 3)(*((w.bnd,) * 3 if isinstance(w.bnd, int) else w.bnd))
        cdp = (C.c_ulonglong * 3)(*[d + 1 for d in w.deg])

        def host_step():
            lib.pull(hf1.data_ptr(), hphi.data_ptr(), hf0.data_ptr(), C.cast(cd0, C.c_void_p), n1,
                     C.cast(cb, C.c_void_p), C.cast(cdp, C.c_void_p), w.ext)
            hacc.zero_()                              # caller zero-fills, src/pushpull_cpu.jl:190
            lib.push(hacc.data_ptr(), hphi.data_ptr(), hf1.data_ptr(), C.cast(cd0, C.c_void_p), n1,
                     C.cast(cb, C.c_void_p), C.cast(cdp, C.c_void_p), w.ext)

        for _ in range(max(args.warmup, 3)):
            host_step()
        if ws > 1:
            dist.barrier()
        te = time.perf_counter()
        for _ in range(args.steps):
            host_step()
        e2e_s = (time.perf_counter() - te) / args.steps
        if ws > 1:
            t = torch.tensor([e2e_s], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            e2e_s = float(t.item())
        e2e = {"value": ws * n1 * nc / e2e_s / 1e9, "unit": "Gvox/s",
               "h2d_bytes_per_step": (12 * n1 + 4 * n0) + (12 * n1 + 4 * n1 + 4 * n0),
               "d2h_bytes_per_step": 4 * n1 + 4 * n0,
               "ms_per_step": e2e_s * 1e3,
               "path": "host-pointer ABI pull() then push() (artifacts/C/pushpull.h signatures)"}

    fused = None if args.no_fused else fused_vs_plain(pkg, dev, args)
    batched = None if args.no_batch else batched_leg(pkg, dev, args)
    contention = None if args.no_contention else contention_leg(pkg, dev, args)

    if rank != 0:
        if ws > 1:
            dist.destroy_process_group()
        return 0

    peak, peak_src = _peaks()
    bytes_pull = 12 * n1 + 4 * nc * n0 + 4 * nc * n1
    bytes_push = 12 * n1 + 4 * nc * n1 + 4 * nc * n0
    mp, mq = statistics.mean(pull_ms), statistics.mean(push_ms)
    dom, dom_ms, dom_bytes = ("push", mq, bytes_push) if mq >= mp else ("pull", mp, bytes_pull)
    ach = dom_bytes / (dom_ms * 1e-3) / 1e9
    roof = {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": peak, "unit": "GB/s",
            "frac": ach / peak, "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)",
            "algorithmic_bytes_per_launch": dom_bytes, "traffic": TRAFFIC.get(dom)}
    kernels = {
        "pull": {"ms": mp, "GB_s": bytes_pull / (mp * 1e-3) / 1e9, "frac_of_peak": bytes_pull / (mp * 1e-3) / 1e9 / peak,
                 "Gvox_s": n1 / (mp * 1e-3) / 1e9},
        "push": {"ms": mq, "GB_s": bytes_push / (mq * 1e-3) / 1e9, "frac_of_peak": bytes_push / (mq * 1e-3) / 1e9 / peak,
                 "Gvox_s": n1 / (mq * 1e-3) / 1e9},
        "pull+push_frac_of_peak": (bytes_pull + bytes_push) / ((mp + mq) * 1e-3) / 1e9 / peak,
    }
    mg = statistics.median(pg_ms)
    bytes_pg = 12 * n1 + 4 * nc * n0 + 12 * nc * n1
    kernels["pull_grad"] = {"ms": mg, "GB_s": bytes_pg / (mg * 1e-3) / 1e9,
                            "frac_of_peak": bytes_pg / (mg * 1e-3) / 1e9 / peak, "Gvox_s": n1 / (mg * 1e-3) / 1e9}
    bytes_pushg = 12 * n1 + 12 * nc * n1 + 4 * nc * n0
    kernels["push_grad"] = {"ms": pushg_ms, "GB_s": bytes_pushg / (pushg_ms * 1e-3) / 1e9,
                            "frac_of_peak": bytes_pushg / (pushg_ms * 1e-3) / 1e9 / peak,
                            "Gvox_s": n1 / (pushg_ms * 1e-3) / 1e9}
    bytes_aff = 4 * nc * n0 + 4 * nc * n1
    for k, ms in (("affine_pull", aff_pull_ms), ("affine_push", aff_push_ms)):
        kernels[k] = {"ms": ms, "GB_s": bytes_aff / (ms * 1e-3) / 1e9,
                      "frac_of_peak": bytes_aff / (ms * 1e-3) / 1e9 / peak, "Gvox_s": n1 / (ms * 1e-3) / 1e9}
    kernels["affine_map"] = [[float(v) for v in row] for row in Aff]
    for k in ("pull", "push", "pull_grad", "push_grad", "affine_pull", "affine_push"):
        kernels[k]["traffic_bytes_ncu"] = TRAFFIC.get(k)
    kernels["bytes_model"] = ("algorithmic bytes per launch: pull 12 n1 (phi) + 4 n0 (image, once) + 4 n1 (out); "
                              "push 12 n1 + 4 n1 (values) + 4 n0 (image written once); pull_grad 12 n1 + 4 n0 + 12 n1; "
                              "push_grad 12 n1 + 12 n1 (gradient) + 4 n0; "
                              "affine pull 4 n0 + 4 n1, affine push 4 n1 + 4 n0 (no deformation)")
    cpu = None
    if not args.no_cpu and ws == 1 or (not args.no_cpu and rank == 0):
        cpu, _ = cpu_baseline(w, seconds=args.cpu_seconds)
    line = {"metric": METRIC, "value": value, "unit": "Gvox/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded): smoothed U(0,1) image, smoothed "
            "random displacement", "config": _config(w, args), "roofline": roof, "cpu_baseline": cpu,
            "e2e": e2e, "gpu_launches": 2 * args.steps, "clocks": clk.summary(), "kernels": kernels,
            "accuracy_vs_fp64": accuracy,
            "fused_step": fused, "batched": batched, "contention_push": contention,
            "wall_s_timed_region": wall}
    print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()
    return 0


def fused_vs_plain(pkg, dev, args):
    """Differentiable step on 160x192x160 (degree 2, bounds (0,1,2)): the fused kernel
    against the plain sequence pull -> pull_grad -> push plus the residual and
    contraction broadcasts (how the reference's pull rrule evaluates it)."""
    import torch
    from pushpull_gb300 import workloads
    L = pkg.layout
    w = workloads.config3(seed=args.seed + 1)
    s = pkg.Settings(w.deg, w.bnd, w.ext)
    f0 = L.from_numpy(w.f0, dev)
    phi = L.from_numpy(w.phi, dev)
    g = pkg.pull(f0, L.from_numpy(w.extra["phi2"], dev), s)
    d0 = tuple(w.f0.shape[:3])
    n1 = int(np.prod(w.phi.shape[:3]))
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def plain():
        f1 = pkg.pull(f0, phi, s)
        gr = pkg.pull_grad(f0, phi, s)                       # (d1, 3)
        r = f1 - g
        loss = (r.double() * r.double()).sum()
        delta = 2 * r
        df = pkg.push(delta, phi, d0, s)
        dphi = gr * delta.unsqueeze(3)                        # sum over the single channel
        return loss, df, dphi

    def fused():
        return pkg.fused_step(f0, phi, g, s)

    def timeit(fn, reps):
        for _ in range(3):
            fn()
        ms = []
        for _ in range(reps):
            _flush(flush)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        return statistics.median(ms)

    reps = max(args.steps, 5)
    t_plain, t_fused = timeit(plain, reps), timeit(fused, reps)
    f1 = pkg.pull(f0, phi, s)
    parts = {"pull": timeit(lambda: pkg.pull(f0, phi, s, out=f1), reps),
             "pull_grad": timeit(lambda: pkg.pull_grad(f0, phi, s), reps),
             "push": timeit(lambda: pkg.push(f1, phi, d0, s), reps)}
    lp, dfp, dpp = plain()
    lf, dff, dpf = fused()

    def rel(a, b):
        a, b = a.double(), b.double()
        return float((a - b).abs().max() / b.abs().max())
    accuracy = None
    if not args.no_accuracy:
        from oracle import oracle as O
        so, th = O.Sett.make(w.deg, w.bnd, w.ext), _oracle_threads()
        gn = L.to_numpy(g)
        r = O.pull(w.f0, w.phi, so, threads=th) - gn
        ref_loss = float(np.sum(r * r))
        d = np.asfortranarray((2 * r).astype(np.float32))
        accuracy = {"loss": abs(float(lf) - ref_loss) / abs(ref_loss),
                    "df": _errors(L.to_numpy(dff), O.push(d, w.phi, d0, so, threads=th)),
                    "dphi": _errors(L.to_numpy(dpf), O.pull_grad(w.f0, w.phi, so, threads=th) * (2 * r)[..., None],
                                    floor=1e-2),
                    "reference": "FP64 oracle on the same inputs, whole volume"}
    bytes_fused = 12 * n1 + 4 * int(np.prod(d0)) + 4 * n1 + 12 * n1 + 4 * int(np.prod(d0))
    return {"workload": "loss = sum((pull(f, phi) - g)^2), 160x192x160 Float32, degree 2, bounds (0,1,2), "
                        "ext=1, g = pull(f, phi2)",
            "plain_ms": t_plain, "fused_ms": t_fused, "speedup": t_plain / t_fused, "plain_kernels_ms": parts,
            "fused_Gvox_s": n1 / (t_fused * 1e-3) / 1e9,
            "fused_GB_s_algorithmic": bytes_fused / (t_fused * 1e-3) / 1e9,
            "rel_diff_fused_vs_plain": {"loss": abs(float(lf) - float(lp)) / abs(float(lp)),
                                        "df": rel(dff, dfp), "dphi": rel(dpf, dpp)},
            "plain": "pull, pull_grad, push kernels + torch residual/reduction/contraction (5 launches + 4 torch ops)",
            "accuracy_vs_fp64": accuracy}


def _timeit(fn, reps, flush):
    import torch
    for _ in range(3):
        fn()
    ms = []
    for _ in range(reps):
        _flush(flush)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    return statistics.median(ms)


def batched_leg(pkg, dev, args):
    """Uneven batch: 32 pairs with sizes from 64^3 to 256x256x192, 1-3 channels,
    degrees from {1,2,3}, each with a 3-level pyramid (96 volumes); pull then push
    of every volume in one persistent launch replayed from a CUDA graph, against
    one pull and one push call per volume."""
    import torch
    from pushpull_gb300 import batch as B
    from pushpull_gb300 import workloads as W
    L = pkg.layout
    specs = W.batched_pairs(seed=4, npairs=32, levels=3)
    items = []
    vox = 0
    for sp in specs:
        d, c = sp["d"], sp["channels"]
        f0 = W.image_gpu(d, sp["seed"], fwhm=3.0, channels=c, device=dev)
        phi = W.deformation_gpu(d, sp["seed"] + 7, fwhm=8.0, amplitude=3.0 / (1 << sp["level"]), device=dev)
        f1 = L.empty(tuple(d) + ((c,) if c > 1 else ()), device=dev)
        out = L.empty(tuple(f0.shape), device=dev)
        items.append(dict(f0=f0, phi=phi, f1=f1, out=out, sett=pkg.Settings(sp["deg"], 1, 1)))
        vox += int(np.prod(d)) * c
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    plan = B.BatchPlan(items, zero_outputs=True)
    with torch.cuda.stream(stream):
        plan.capture(stream)
    torch.cuda.synchronize()

    def graph():
        stream.wait_stream(torch.cuda.current_stream())
        plan.launch(stream)
        torch.cuda.current_stream().wait_stream(stream)

    def per_item():
        for it in items:
            pkg.pull(it["f0"], it["phi"], it["sett"], out=it["f1"])
            pkg.push(it["f1"], it["phi"], tuple(it["f0"].shape[:3]), it["sett"], out=it["out"], accumulate=False)

    reps = max(min(args.steps, 10), 3)
    t_graph = _timeit(graph, reps, flush)
    t_items = _timeit(per_item, reps, flush)
    tiles = plan.tiles
    plan.close()
    return {"workload": "32 pairs x 3 pyramid levels (96 volumes), sizes U[64,256]x[64,256]x[64,192] halved per "
                        "level, 1-3 channels, degree from {1,2,3}, DCT-II, ext=1; pull then push each",
            "voxels_x_channels": vox, "tiles": tiles, "graph_ms": t_graph, "per_item_ms": t_items,
            "graph_Gvox_s": vox / (t_graph * 1e-3) / 1e9, "per_item_Gvox_s": vox / (t_items * 1e-3) / 1e9,
            "speedup_vs_per_item": t_items / t_graph,
            "launches": {"graph": 1, "per_item": 2 * len(items)}}


def contention_leg(pkg, dev, args):
    """Many-to-one scatter: 256^3 x 3 channels, cubic, DCT-II, deformation = 0.25x
    contraction about the centre + FWHM-12 field of +-3 vox; push and push_grad."""
    import torch
    from pushpull_gb300 import workloads as W
    L = pkg.layout
    d = (256, 256, 256)
    s = pkg.Settings(3, 1, 1)
    f1 = W.image_gpu(d, 51, fwhm=3.0, channels=3, device=dev)
    g1 = L.empty(d + (3, 3), device=dev)
    g1.copy_(torch.randn(g1.shape, generator=torch.Generator(device=dev).manual_seed(52), device=dev))
    phi = W.deformation_gpu(d, 53, fwhm=12.0, amplitude=3.0, contraction=0.25, device=dev)
    out = L.empty(d + (3,), device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    reps = max(min(args.steps, 10), 3)
    t_push = _timeit(lambda: pkg.push(f1, phi, d, s, out=out, accumulate=False), reps, flush)
    t_pushg = _timeit(lambda: pkg.push_grad(g1, phi, d, s, out=out, accumulate=False), reps, flush)
    n1, nc = int(np.prod(d)), 3
    taps = 64
    accuracy = None
    if not args.no_accuracy:
        from oracle import oracle as O
        so, th = O.Sett.make(3, 1, 1), _oracle_threads()
        pn = L.to_numpy(phi)
        accuracy = {"push": _errors(L.to_numpy(pkg.push(f1, phi, d, s)),
                                    O.push(L.to_numpy(f1), pn, d, so, threads=th)),
                    "push_grad": _errors(L.to_numpy(pkg.push_grad(g1, phi, d, s)),
                                         O.push_grad(L.to_numpy(g1), pn, d, so, threads=th), floor=1e-2),
                    "reference": "FP64 oracle on the same inputs, whole volume"}
    return {"workload": "push and push_grad, 256^3 x 3 channels Float32, cubic, DCT-II, ext=1, phi = 0.25x "
                        "contraction about the centre + FWHM-12 field +-3 vox (source occupies ~1/64 of the grid)",
            "push_ms": t_push, "push_grad_ms": t_pushg,
            "push_Gvox_s": n1 * nc / (t_push * 1e-3) / 1e9, "push_grad_Gvox_s": n1 * nc / (t_pushg * 1e-3) / 1e9,
            "scatter_updates_per_s": {"push": n1 * nc * taps / (t_push * 1e-3),
                                      "push_grad": n1 * nc * taps / (t_pushg * 1e-3)},
            "note": "scatter updates = voxels x channels x 64 taps, accumulated in shared memory as fixed-point "
                    "integers (privatised) and flushed to HBM once per box word",
            "accuracy_vs_fp64": accuracy}


PROFILE_CASES = ("pull", "pull_grad", "push", "affine_pull", "affine_push", "contention_push",
                 "contention_push_grad", "fused", "nearest_pull", "pull_hess_dot")


def run_profile(args):
    """Launch one op on its benchmark workload --warmup + --steps times, untimed:
    the program the ncu captures run (192^3 cubic for pull, pull_grad, push,
    pull_hess_dot and the affine ops; the same deformation at degree 0 for
    nearest_pull; the 256^3 x 3 contraction for contention_*; the 160x192x160
    quadratic step for fused)."""
    import torch
    import __graft_entry__ as entry
    from pushpull_gb300 import workloads as W
    pkg = entry.package()
    L = pkg.layout
    dev = torch.device("cuda", 0)
    case = args.profile
    if case.startswith("contention"):
        d = (256, 256, 256)
        s = pkg.Settings(3, 1, 1)
        phi = W.deformation_gpu(d, 53, fwhm=12.0, amplitude=3.0, contraction=0.25, device=dev)
        out = L.empty(d + (3,), device=dev)
        if case == "contention_push":
            f1 = W.image_gpu(d, 51, fwhm=3.0, channels=3, device=dev)
            fn = lambda: pkg.push(f1, phi, d, s, out=out, accumulate=False)   # noqa: E731
        else:
            g1 = L.empty(d + (3, 3), device=dev)
            g1.copy_(torch.randn(g1.shape, generator=torch.Generator(device=dev).manual_seed(52), device=dev))
            fn = lambda: pkg.push_grad(g1, phi, d, s, out=out, accumulate=False)   # noqa: E731
    elif case == "fused":
        w = W.config3(seed=args.seed + 1)
        s = pkg.Settings(w.deg, w.bnd, w.ext)
        f0, phi = L.from_numpy(w.f0, dev), L.from_numpy(w.phi, dev)
        g = pkg.pull(f0, L.from_numpy(w.extra["phi2"], dev), s)
        fn = lambda: pkg.fused_step(f0, phi, g, s)   # noqa: E731
    else:
        w = _workload(args)
        s = pkg.Settings(w.deg, w.bnd, w.ext)
        d0, d1 = tuple(w.f0.shape[:3]), tuple(w.phi.shape[:3])
        f0, phi = L.from_numpy(w.f0, dev), L.from_numpy(w.phi, dev)
        f1 = pkg.pull(f0, phi, s)
        Aff = W.affine_map(d0, seed=args.seed + 4)
        out0, out1, outg = L.empty(d0, device=dev), L.empty(d1, device=dev), L.empty(d1 + (3,), device=dev)
        s0 = pkg.Settings(0, w.bnd, w.ext)
        up = L.empty(d1 + (3,), device=dev)
        up.copy_(torch.randn(up.shape, generator=torch.Generator(device=dev).manual_seed(54), device=dev))
        fn = {"pull": lambda: pkg.pull(f0, phi, s, out=out1),
              "nearest_pull": lambda: pkg.pull(f0, phi, s0, out=out1),
              "pull_hess_dot": lambda: pkg.pull_hess_dot(f0, phi, up, s),
              "pull_grad": lambda: pkg.pull_grad(f0, phi, s, out=outg),
              "push": lambda: pkg.push(f1, phi, d0, s, out=out0, accumulate=False),
              "affine_pull": lambda: pkg.affine_pull(f0, Aff, d1, s, out=out1),
              "affine_push": lambda: pkg.affine_push(f1, Aff, d0, s, out=out0)}[case]
    for _ in range(args.warmup + args.steps):
        fn()
    torch.cuda.synchronize()
    status = int(pkg.native_library().pp_device_status(1))
    print(json.dumps({"profile": case, "launches": args.warmup + args.steps, "device_status": status}))
    return 0 if status == 0 else 1


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=8.0)
    ap.add_argument("--no-fused", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-contention", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the FP64 error fields")
    ap.add_argument("--profile", choices=PROFILE_CASES, default=None,
                    help="launch one op warmup + steps times without timing (for ncu captures)")
    args = ap.parse_args(argv)
    import __graft_entry__ as entry
    entry.package()
    if args.profile:
        return run_profile(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
