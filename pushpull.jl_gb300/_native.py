"""ctypes binding of ``lib/libpushpull_gb300.so`` (the C ABI in include/pushpull_gb300.h).

There is no fallback: if the library is missing or cannot be loaded every op
raises.  Build it with ``__graft_entry__.build()`` or ``python pushpull.jl_gb300/build.py``.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib: C.CDLL | None = None

PP_STATUS = {
    0: "PP_OK", 1: "PP_ERR_NULL", 2: "PP_ERR_DIMS", 3: "PP_ERR_DEGREE", 4: "PP_ERR_BOUND",
    5: "PP_ERR_CHANNELS", 6: "PP_ERR_ALIGN", 7: "PP_ERR_CUDA", 8: "PP_ERR_UNSUPPORTED",
    9: "PP_ERR_TOO_LARGE", 10: "PP_ERR_TIMEOUT",
}

_u64x3 = C.c_ulonglong * 3
_i32x3 = C.c_int * 3
_vp = C.c_void_p

class BatchItem(C.Structure):
    """pp_batch_item of include/pushpull_gb300.h."""
    _fields_ = [("f0", _vp), ("phi", _vp), ("f1", _vp), ("out", _vp), ("d0", C.c_ulonglong * 3),
                ("d1", C.c_ulonglong * 3), ("nc", C.c_int), ("deg", C.c_int), ("bnd", C.c_int * 3),
                ("ext", C.c_int), ("deg3", C.c_int * 3), ("nbnd", C.c_int), ("bnds", _vp)]


# name -> (restype, argtypes)
_SIGS = {
    "pp_pull": (C.c_int, [_vp, _vp, _vp, _u64x3, _u64x3, C.c_int, C.c_int, _vp, C.c_int, _i32x3,
                          C.c_int, _vp]),
    "pp_pull_grad": (C.c_int, [_vp, _vp, _vp, _u64x3, _u64x3, C.c_int, C.c_int, _vp, C.c_int,
                               _i32x3, C.c_int, _vp]),
    "pp_pull_hess": (C.c_int, [_vp, _vp, _vp, _u64x3, _u64x3, C.c_int, C.c_int, _vp, C.c_int,
                               _i32x3, C.c_int, _vp]),
    "pp_pull_grad_dot": (C.c_int, [_vp, _vp, _vp, _vp, _u64x3, _u64x3, C.c_int, C.c_int, _vp, C.c_int,
                                   _i32x3, C.c_int, _vp]),
    "pp_pull_hess_dot": (C.c_int, [_vp, _vp, _vp, _vp, _u64x3, _u64x3, C.c_int, C.c_int, _vp, C.c_int,
                                   _i32x3, C.c_int, _vp]),
    "pp_push": (C.c_int, [_vp, _vp, _vp, _u64x3, _u64x3, C.c_int, C.c_int, _vp, C.c_int, _i32x3,
                          C.c_int, C.c_int, _vp]),
    "pp_push_grad": (C.c_int, [_vp, _vp, _vp, _u64x3, _u64x3, C.c_int, C.c_int, _vp, C.c_int,
                               _i32x3, C.c_int, C.c_int, _vp]),
    "pp_fused_step": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _u64x3, _u64x3, C.c_int, C.c_int, _vp, C.c_int,
                                _i32x3, C.c_int, C.c_int, _vp]),
    "pp_push_count": (C.c_int, [_vp, _vp, _vp, _vp, _u64x3, _u64x3, C.c_int, C.c_int, _vp, C.c_int, _i32x3,
                                C.c_int, C.c_int, _vp]),
    "pp_fused_step_noalloc": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _u64x3, _u64x3, C.c_int, C.c_int, _vp,
                                        C.c_int, _i32x3, C.c_int, C.c_int, _vp]),
    "pp_pull_affine": (C.c_int, [_vp, _vp, _vp, _u64x3, _u64x3, C.c_int, C.c_int, _vp, C.c_int, _i32x3, C.c_int,
                                 _vp]),
    "pp_push_affine": (C.c_int, [_vp, _vp, _vp, _u64x3, _u64x3, C.c_int, C.c_int, _vp, C.c_int, _i32x3, C.c_int,
                                 C.c_int, _vp]),
    "pp_batch_create": (C.c_int, [C.POINTER(_vp), C.POINTER(BatchItem), C.c_int, C.c_int]),
    "pp_batch_tiles": (C.c_int, [_vp]),
    "pp_batch_run": (C.c_int, [_vp, _vp]),
    "pp_batch_capture": (C.c_int, [_vp, _vp]),
    "pp_batch_launch": (C.c_int, [_vp, _vp]),
    "pp_batch_destroy": (None, [_vp]),
    "pp_autotune": (C.c_int, [C.c_int, _vp, _vp, _vp, _u64x3, _u64x3, C.c_int, C.c_int, _vp, C.c_int, _i32x3,
                              C.c_int, C.c_int, _vp, C.POINTER(C.c_int), C.POINTER(C.c_float)]),
    "pp_last_error": (C.c_char_p, []),
    "pp_set_tile": (C.c_int, [C.c_int] * 6),
    "pp_get_tile": (C.c_int, [C.c_int, C.c_int] + [C.POINTER(C.c_int)] * 4),
    "pp_set_path": (C.c_int, [C.c_int]),
    "pp_version": (C.c_int, []),
    "pp_device_status": (C.c_uint, [C.c_int]),
    "pp_test_bounded_wait": (C.c_int, [C.c_longlong, _vp]),
    # compatibility layer: reference CPU signatures on host pointers
    "pull": (None, [_vp, _vp, _vp, _vp, C.c_ulonglong, _vp, _vp, C.c_int]),
    "pullg": (None, [_vp, _vp, _vp, _vp, C.c_ulonglong, _vp, _vp, C.c_int]),
    "pullh": (None, [_vp, _vp, _vp, _vp, C.c_ulonglong, _vp, _vp, C.c_int]),
    "push": (None, [_vp, _vp, _vp, _vp, C.c_ulonglong, _vp, _vp, C.c_int]),
    "pushg": (None, [_vp, _vp, _vp, _vp, C.c_ulonglong, _vp, _vp, C.c_int]),
}


class PushPullError(RuntimeError):
    def __init__(self, fn: str, code: int, msg: str):
        super().__init__(f"{fn}: {PP_STATUS.get(code, code)}: {msg}")
        self.code = code


def library_path() -> str:
    return _build.LIB


def lib() -> C.CDLL:
    """Load (once) the native library; raises if it has not been built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not os.path.exists(path):
            raise RuntimeError(f"pushpull_gb300 native library not built: {path} is missing "
                               "(run __graft_entry__.build())")
        so = C.CDLL(path)
        for name, (res, args) in _SIGS.items():
            fn = getattr(so, name)
            fn.restype = res
            fn.argtypes = args
        _lib = so
        return so


def declared_symbols() -> list[str]:
    return list(_SIGS)


def check(fn: str, rc: int) -> None:
    if rc != 0:
        msg = lib().pp_last_error()
        raise PushPullError(fn, rc, msg.decode() if msg else "")


def u64x3(v) -> "C.Array":
    return _u64x3(*[int(x) for x in v])


def i32x3(v) -> "C.Array":
    return _i32x3(*[int(x) for x in v])
