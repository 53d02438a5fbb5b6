"""pushpull_gb300 -- GB300-native B-spline pull / push (PushPull.jl's resampling hot path).

Host-side mirror of the reference API (src/PushPull.jl:19-20 exports) over the
C ABI of ``lib/libpushpull_gb300.so`` (include/pushpull_gb300.h).
"""
from . import autograd, layout
from ._native import PushPullError, lib as native_library
from .api import (adjust_affine, affine_pull, affine_push, fused_step, id, pull, pull_grad, pull_grad_dot,
                  pull_hess, pull_hess_dot, push, push_count, push_grad)
from .compositions import Exp, ExpPlan, compose
from .settings import Settings, sett_chan

__all__ = [
    "Settings", "sett_chan", "pull", "pull_grad", "pull_hess", "push", "push_grad", "id",
    "pull_grad_dot", "pull_hess_dot", "fused_step", "affine_pull", "affine_push", "adjust_affine",
    "push_count", "compose", "Exp", "ExpPlan",
    "autograd", "layout", "PushPullError",
    "native_library",
]
