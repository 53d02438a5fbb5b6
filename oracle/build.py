"""Build recipe for the CPU checkers (test infrastructure only).

* ``lib/libpp_oracle.so``  -- the FP64 oracle and FP32 port from ``pp_oracle.c``.
* ``_ref/libpp_ref.so``    -- the reference's own CPU library, compiled from its
  C sources (``artifacts/C/pushpull.c``, which #includes ``pushpull_dev.cu``,
  ``bspline.cu`` and ``patch.cu``).  The flags keep float contraction off so the
  build does what the source says.

Where the reference tree is present (its location is ``$PP_REFERENCE_DIR``,
default ``/root/reference``), ``stage_ref_sources`` copies those five files,
unmodified, into ``_ref/src/``.  ``_ref/`` is kept out of version control but
travels with the working copy, so a host without the reference tree (the GPU
machine) compiles the same sources with its own compiler; no binary moves
between hosts.  Nothing here is used by the shipped library.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "lib", "libpp_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_SO = os.path.join(REF_DIR, "libpp_ref.so")
REF_STAGE = os.path.join(REF_DIR, "src")
REF_DEPS = ("pushpull.c", "pushpull_dev.cu", "bspline.cu", "patch.cu", "cuheader.h")

CC = os.environ.get("CC", "gcc")


def reference_src_dir() -> str:
    """The reference's ``artifacts/C`` directory (``$PP_REFERENCE_DIR``, default /root/reference)."""
    return os.path.join(os.environ.get("PP_REFERENCE_DIR", "/root/reference"), "artifacts", "C")


def _stale(target: str, sources) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources if os.path.exists(s))


def oracle_cmd() -> list[str]:
    return [CC, "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", ORACLE_SO,
            os.path.join(HERE, "pp_oracle.c"), "-lm"]


def ref_cmd(src_dir: str) -> list[str]:
    return [CC, "-O3", "-ffp-contract=off", "-fPIC", "-shared", "-o", REF_SO,
            os.path.join(src_dir, "pushpull.c"), "-lm"]


def build_oracle(force: bool = False) -> str:
    srcs = [os.path.join(HERE, "pp_oracle.c"), os.path.join(HERE, "pp_oracle.h")]
    if force or _stale(ORACLE_SO, srcs):
        os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
        subprocess.run(oracle_cmd(), check=True)
    return ORACLE_SO


def reference_present() -> bool:
    return all(os.path.exists(os.path.join(reference_src_dir(), f)) for f in REF_DEPS)


def stage_ref_sources() -> bool:
    """Copy the reference's five C sources into ``_ref/src`` (when the tree is here)."""
    if not reference_present():
        return False
    os.makedirs(REF_STAGE, exist_ok=True)
    for f in REF_DEPS:
        src, dst = os.path.join(reference_src_dir(), f), os.path.join(REF_STAGE, f)
        if _stale(dst, [src]):
            shutil.copyfile(src, dst)
    return True


def _staged() -> bool:
    return all(os.path.exists(os.path.join(REF_STAGE, f)) for f in REF_DEPS)


def build_ref(force: bool = False) -> str | None:
    """Compile the reference CPU library from its sources; None when neither the
    reference tree nor a staged copy of its sources is available."""
    stage_ref_sources()
    if not _staged():
        return None
    deps = [os.path.join(REF_STAGE, f) for f in REF_DEPS]
    if force or _stale(REF_SO, deps):
        subprocess.run(ref_cmd(REF_STAGE), check=True)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
