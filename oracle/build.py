"""Build recipe for the CPU checkers (test infrastructure only).

* ``lib/libpp_oracle.so``  -- the FP64 oracle and FP32 port from ``pp_oracle.c``.
* ``_ref/libpp_ref.so``    -- the reference's own CPU library, compiled from its
  C sources (``artifacts/C/pushpull.c``, which #includes ``pushpull_dev.cu``,
  ``bspline.cu`` and ``patch.cu``) wherever the reference tree is present.  The
  flags keep float contraction off so the build does what the source says.

Nothing here is used by the shipped library.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "lib", "libpp_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libpp_ref.so")
REF_SRC_DIR = "/root/reference/artifacts/C"
REF_SRC = os.path.join(REF_SRC_DIR, "pushpull.c")
REF_DEPS = ("pushpull.c", "pushpull_dev.cu", "bspline.cu", "patch.cu", "cuheader.h")

CC = os.environ.get("CC", "gcc")


def _stale(target: str, sources) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources if os.path.exists(s))


def oracle_cmd() -> list[str]:
    return [CC, "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", ORACLE_SO,
            os.path.join(HERE, "pp_oracle.c"), "-lm"]


def ref_cmd() -> list[str]:
    return [CC, "-O3", "-ffp-contract=off", "-fPIC", "-shared", "-o", REF_SO, REF_SRC, "-lm"]


def build_oracle(force: bool = False) -> str:
    srcs = [os.path.join(HERE, "pp_oracle.c"), os.path.join(HERE, "pp_oracle.h")]
    if force or _stale(ORACLE_SO, srcs):
        os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
        subprocess.run(oracle_cmd(), check=True)
    return ORACLE_SO


def reference_present() -> bool:
    return os.path.exists(REF_SRC)


def build_ref(force: bool = False) -> str | None:
    """Compile the reference CPU library from source; None when the tree is absent."""
    if not reference_present():
        return REF_SO if os.path.exists(REF_SO) else None
    deps = [os.path.join(REF_SRC_DIR, f) for f in REF_DEPS]
    if force or _stale(REF_SO, deps):
        os.makedirs(os.path.dirname(REF_SO), exist_ok=True)
        subprocess.run(ref_cmd(), check=True)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
