"""Build ``lib/libpushpull_gb300.so`` from ``csrc/*.cu`` with nvcc for sm_103a.

Each translation unit compiles in parallel; the shared library links the CUDA
runtime statically so that any host (Python ctypes, Julia ``ccall``) can load it
without extra search paths.  Rebuilds only when a source or header changed.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIB = os.path.join(LIBDIR, "libpushpull_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-v",
              "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _headers():
    return sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h")))


def _obj(src: str) -> str:
    return os.path.join(OBJDIR, os.path.basename(src)[:-3] + ".o")


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJDIR, exist_ok=True)
    headers = _headers()
    srcs = _sources()
    todo = [s for s in srcs if force or _newer(_obj(s), [s] + headers)]

    def compile_one(src):
        cmd = [nvcc()] + ARCH + NVCC_FLAGS + ["-c", src, "-o", _obj(src)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        log = _obj(src)[:-2] + ".ptxas.log"
        with open(log, "w") as fh:
            fh.write(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stderr[-4000:]}")
        return src

    if todo:
        with ThreadPoolExecutor(max_workers=min(len(todo), os.cpu_count() or 4)) as ex:
            for s in ex.map(compile_one, todo):
                if verbose:
                    print("compiled", os.path.basename(s), file=sys.stderr)
    objs = [_obj(s) for s in srcs]
    if force or todo or _newer(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs
        subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
