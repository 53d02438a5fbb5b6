"""pushpull_gb300 -- GB300-native B-spline pull / push (PushPull.jl's resampling hot path).

Host-side mirror of the reference API (src/PushPull.jl:19-20 exports) over the
C ABI of ``lib/libpushpull_gb300.so`` (include/pushpull_gb300.h).
"""
from . import layout
from ._native import PushPullError, lib as native_library
from .api import id, pull, pull_grad, pull_hess, push, push_grad
from .settings import Settings, sett_chan

__all__ = [
    "Settings", "sett_chan", "pull", "pull_grad", "pull_hess", "push", "push_grad", "id",
    "layout", "PushPullError", "native_library",
]
