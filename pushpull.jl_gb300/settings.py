"""``Settings`` -- the push/pull configuration, mirroring src/pushpull_general.jl:15-60.

* ``deg``  per-dimension B-spline degree, clamped to 0..4 (an int applies to all three);
* ``bnd``  boundary codes 0 circulant, 1 reflect (DCT-II), 2 antisymmetric
  reflect (DST-II): an int, a 3-tuple, a list of 3-tuples (one per channel) or a
  3 x C matrix; every code must be in {0, 1, 2};
* ``ext``  extrapolate flag, clamped to 0/1.

Defaults as the reference: ``Settings()`` = degree 1, reflect, extrapolate.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

_ALLOWED = (0, 1, 2)


@dataclass(frozen=True)
class Settings:
    deg: tuple = (1, 1, 1)
    bnd: tuple = ((1, 1, 1),)
    ext: int = 1
    _packed: tuple = field(default=(), compare=False, repr=False)

    def __init__(self, deg=(1, 1, 1), bnd=((1, 1, 1),), ext=True):
        if isinstance(deg, (int, np.integer)):
            deg = (deg, deg, deg)
        deg = tuple(int(max(min(int(d), 4), 0)) for d in deg)
        assert len(deg) == 3
        if isinstance(bnd, (int, np.integer)):
            assert int(bnd) in _ALLOWED
            bnd1 = ((int(bnd),) * 3,)
        elif isinstance(bnd, np.ndarray) and bnd.ndim == 2:
            assert bnd.shape[0] == 3
            assert all(int(v) in _ALLOWED for v in bnd.ravel())
            bnd1 = tuple(tuple(int(v) for v in bnd[:, i]) for i in range(bnd.shape[1]))
        elif isinstance(bnd, (list, tuple)) and len(bnd) > 0 and isinstance(bnd[0], (list, tuple, np.ndarray)):
            bnd1 = []
            for b in bnd:
                assert len(b) == 3 and all(int(v) in _ALLOWED for v in b)
                bnd1.append(tuple(int(v) for v in b))
            bnd1 = tuple(bnd1)
        else:
            assert len(bnd) == 3 and all(int(v) in _ALLOWED for v in bnd)
            bnd1 = (tuple(int(v) for v in bnd),)
        ext = int(max(min(int(ext), 1), 0))
        object.__setattr__(self, "deg", deg)
        object.__setattr__(self, "bnd", bnd1)
        object.__setattr__(self, "ext", ext)
        flat = [v for b in bnd1 for v in b]
        object.__setattr__(self, "_packed", tuple(flat))

    # ---- helpers used by the C-ABI calls ------------------------------------
    @property
    def nbnd(self) -> int:
        return len(self.bnd)

    def bnd_array(self) -> "C.Array":
        return (C.c_int * len(self._packed))(*self._packed)

    def for_channel(self, c: int) -> "Settings":
        """Settings of one channel (``sett_chan``, src/pushpull_general.jl:63-69)."""
        b = self.bnd[0] if len(self.bnd) == 1 else self.bnd[c]
        return Settings(self.deg, b, self.ext)


def sett_chan(sett: Settings, c: int) -> Settings:
    return sett.for_channel(c)
