"""Host logic without a GPU: Settings (src/pushpull_general.jl:15-60) and the
column-major layout helpers."""
from __future__ import annotations

import numpy as np
import pytest
import torch


def test_settings_defaults_and_clamping(pkg):
    s = pkg.Settings()
    assert s.deg == (1, 1, 1) and s.bnd == ((1, 1, 1),) and s.ext == 1
    s = pkg.Settings(7, 0, 5)
    assert s.deg == (4, 4, 4) and s.bnd == ((0, 0, 0),) and s.ext == 1
    s = pkg.Settings((-2, 3, 9), (0, 1, 2), 0)
    assert s.deg == (0, 3, 4) and s.bnd == ((0, 1, 2),) and s.ext == 0
    s = pkg.Settings(2, [(0, 0, 0), (1, 2, 1)], -3)
    assert s.nbnd == 2 and s.ext == 0
    assert s.for_channel(1).bnd == ((1, 2, 1),)
    m = np.array([[0, 1], [1, 2], [2, 0]])
    assert pkg.Settings(1, m).bnd == ((0, 1, 2), (1, 2, 0))
    assert list(pkg.Settings(1, [(0, 1, 2), (2, 1, 0)]).bnd_array()) == [0, 1, 2, 2, 1, 0]


@pytest.mark.parametrize("bad", [3, (0, 1, 3), [(0, 1, 2), (4, 0, 0)], -1])
def test_settings_rejects_bad_boundaries(pkg, bad):
    with pytest.raises(AssertionError):
        pkg.Settings(1, bad)


def test_layout_roundtrip(pkg):
    L = pkg.layout
    a = np.asfortranarray(np.arange(2 * 3 * 4 * 5, dtype=np.float32).reshape((2, 3, 4, 5), order="F"))
    t = L.from_numpy(a, device=None)
    assert tuple(t.shape) == a.shape and L.is_colmajor(t)
    assert np.array_equal(L.to_numpy(t), a)
    # column-major flat order equals numpy's Fortran ravel
    assert np.array_equal(t.permute(3, 2, 1, 0).reshape(-1).numpy(), a.ravel(order="F"))
    r = L.reshape(t, (6, 20))
    assert np.array_equal(L.to_numpy(r), a.reshape((6, 20), order="F"))
    c = L.colmajor(torch.zeros(3, 4))          # row-major input gets a column-major copy
    assert L.is_colmajor(c)
    assert L.jsize(t, 5) == 1 and L.jsize(t, 2) == 3
