"""The timeout path of the bounded device-side waits, driven to its limit
without faulting or hanging the GPU: one warp waits on a shared-memory barrier
that nothing completes, gives up after a short cycle limit, records bit 0 of
the device status word and returns.  The status must be readable and
clearable afterwards and the context must still run kernels."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_reports(pkg, O):
    lib = pkg.native_library()
    assert lib.pp_device_status(1) == 0                      # clean before
    stream = torch.cuda.current_stream().cuda_stream
    assert lib.pp_test_bounded_wait(200_000, stream) == 0    # ~0.1 ms at 2 GHz
    torch.cuda.synchronize()
    st = lib.pp_device_status(0)
    assert st != 0xFFFFFFFF and st & 1, st                  # the wait gave up and said so
    assert lib.pp_device_status(1) & 1                       # read and clear
    assert lib.pp_device_status(0) == 0                      # cleared
    # the context is intact: an ordinary call still matches the oracle
    L = pkg.layout
    rng = np.random.default_rng(5)
    d = (20, 18, 16)
    f0 = np.asfortranarray(rng.random(d).astype(np.float32))
    phi = np.asfortranarray((O.identity(d) + rng.standard_normal(d + (3,))).astype(np.float32))
    s = pkg.Settings(3, 1, 1)
    got = L.to_numpy(pkg.pull(L.from_numpy(f0), L.from_numpy(phi), s))
    assert rel_err(got, O.pull(f0, phi, O.Sett.make(3, 1, 1))) <= 1e-5
    assert lib.pp_device_status(0) == 0


def test_bounded_wait_rejects_bad_limits(pkg):
    lib = pkg.native_library()
    assert lib.pp_test_bounded_wait(0, None) == 8            # PP_ERR_UNSUPPORTED
    assert lib.pp_test_bounded_wait((1 << 31) + 1, None) == 8
    assert b"limit_cycles" in lib.pp_last_error()
