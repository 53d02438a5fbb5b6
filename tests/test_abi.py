"""The C ABI: the library loads and exports every symbol include/pushpull_gb300.h
declares, and host-side validation rejects bad arguments before any CUDA call
(so these run without a GPU)."""
from __future__ import annotations

import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "pushpull_gb300.h")


def _declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_parses():
    names = _declared()
    for want in ("pp_pull", "pp_pull_grad", "pp_pull_hess", "pp_push", "pp_push_grad",
                 "pp_last_error", "pp_version", "pull", "pullg", "pullh", "push", "pushg"):
        assert want in names


def test_library_exports_declared_symbols(pkg):
    lib = pkg.native_library()
    for name in _declared():
        assert hasattr(lib, name), name
    assert lib.pp_version() >= 100


def test_julia_binding_uses_declared_symbols():
    """Every library symbol the Julia drop-in module calls is declared in the header
    (the module itself needs Julia and CUDA.jl, which this suite does not run)."""
    jl = open(os.path.join(ROOT, "pushpull.jl_gb300", "julia", "PushPullGB300.jl")).read()
    used = set(re.findall(r"_sym\(:(\w+)\)", jl)) | set(re.findall(r":(pp_\w+)", jl))
    assert {"pp_pull", "pp_push", "pp_fused_step", "pp_pull_grad_dot", "pp_last_error"} <= used
    assert used <= set(_declared()), used - set(_declared())


def _call_pull(lib, deg=(1, 1, 1), bnd=(1, 1, 1), nbnd=1, nc=1, nb=1, d0=(4, 4, 4), d1=(3, 3, 3),
               ptr=8):
    b = (C.c_int * len(bnd))(*bnd)
    return lib.pp_pull(C.c_void_p(ptr), C.c_void_p(ptr), C.c_void_p(ptr), (C.c_ulonglong * 3)(*d0),
                       (C.c_ulonglong * 3)(*d1), nc, nb, C.cast(b, C.c_void_p), nbnd,
                       (C.c_int * 3)(*deg), 1, None)


@pytest.mark.parametrize("kw,code", [
    (dict(deg=(5, 1, 1)), 3),
    (dict(deg=(-1, 1, 1)), 3),
    (dict(bnd=(3, 1, 1)), 4),
    (dict(nc=0), 5),
    (dict(nc=2, bnd=(1, 1, 1, 0, 0, 0, 2, 2, 2), nbnd=3), 5),
    (dict(ptr=0), 1),
    (dict(ptr=6), 6),
    (dict(d0=(0, 4, 4)), 2),
])
def test_validation_errors(pkg, kw, code):
    lib = pkg.native_library()
    rc = _call_pull(lib, **kw)
    assert rc == code
    assert lib.pp_last_error().decode()


def test_empty_sample_grid_is_noop(pkg):
    lib = pkg.native_library()
    assert _call_pull(lib, d1=(0, 5, 5), ptr=0) == 0
    assert lib.pp_last_error().decode() == ""


def test_native_errors_raise(pkg):
    import torch
    L = pkg.layout
    s = pkg.Settings(1, 1, 1)
    with pytest.raises(AssertionError, match="three channels"):
        pkg.pull(L.zeros((4, 4, 4), device="cpu"), L.zeros((4, 4, 4, 2), device="cpu"), s)
    with pytest.raises(TypeError, match="CUDA"):
        pkg.pull(L.zeros((4, 4, 4), device="cpu"), L.zeros((4, 4, 4, 3), device="cpu"), s)
    assert torch.float32 == L.zeros((2, 2, 2), device="cpu").dtype


def test_default_kernel_routing(pkg):
    """The tile registry's defaults, per (op, degree): op 0 pull, 1 pull_grad (and
    pull_grad_dot), 2 pull_hess (and pull_hess_dot), 3 push, 4 push_grad, 5 the
    fused step.  (3, 3, 4) selects the warp-specialised pull family, cap 0 the
    per-voxel kernels (the nearest-neighbour kernel for pull at degree 0), other
    shapes the block-synchronous tiled kernels with that box budget."""
    lib = pkg.native_library()

    def tile(op, deg):
        v = [C.c_int() for _ in range(4)]
        assert lib.pp_get_tile(op, deg, *[C.byref(x) for x in v]) == 0
        return tuple(x.value for x in v)

    ws = (3, 3, 4, 15360)
    for op in (0, 1, 2):
        assert tile(op, 0)[3] == 0
        for deg in (1, 2, 3, 4):
            assert tile(op, deg) == ws, (op, deg)
    for op in (3, 4, 5):
        assert tile(op, 0)[3] == 0 and tile(op, 1)[3] == 0, op
    for op in (3, 4):
        for deg in (2, 3, 4):
            assert tile(op, deg) == (3, 3, 3, 16384), (op, deg)
    assert tile(5, 2) == (3, 3, 3, 2560)
    assert tile(5, 3) == (3, 3, 3, 4096) and tile(5, 4) == (3, 3, 3, 4096)
