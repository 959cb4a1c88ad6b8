"""The allocation-free entry point chf_diagnostics_static, through the C ABI.

It exists for callers that cannot allocate device memory (a pool owned by
another runtime, memory committed to the resident state, or a time loop that
must avoid cudaMalloc/cudaFree).  It must agree with chf_diagnostics, the
entry point that reduces into handle-owned scratch, on the same device
arrays, on two calls in a row (the shared static scratch keeps the previous
call's values, so the second call checks that nothing stale leaks in).
This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

from channel_flow_gb300 import Channel, config, fields
from channel_flow_gb300.channel import CDiag

pytestmark = pytest.mark.gpu


def _dev(ch, which):
    p = ctypes.c_void_p()
    assert ch.L.chf_device_field(ch.h, which, ctypes.byref(p)) == 0
    return p


@pytest.mark.parametrize("seed", [0, 1])
def test_static_diagnostics_match_handle_diagnostics(chflow_lib, seed):
    cfg = config.small(nnx=24, nny=12, nnz=20, aphi=1.5, beta=0.75, dt=5e-4, re=300.0, re_p=1.0)
    st = fields.reference_like_state(cfg, seed=seed, epsilon=0.3, noise=0.02, gamma=5.0)
    with Channel(cfg) as ch:
        ch.upload_state(st)
        ch.getnonlinear()
        ch.solve()
        ch.synchronize()
        ref = ch.diagnostics()
        # field slots: 0 vnp1, 1 omegaynp1, 2 unp1, 3 wnp1, 4 omegaxnp1, 5 omegaznp1
        ptrs = [_dev(ch, i) for i in (2, 0, 3, 4, 1, 5)]
        for _ in range(2):
            prof = np.zeros(cfg.nnz + 1)
            d = CDiag()
            rc = chflow_lib.chf_diagnostics_static(
                cfg.nnx, cfg.nny, cfg.nnz, *ptrs,
                prof.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(d), None)
            assert rc == 0
            assert d.finite == 1
            assert abs(d.energy - ref["energy"]) <= 1e-12 * ref["energy"]
            assert d.max_abs == ref["max_abs"]
            assert abs(prof.sum() - d.energy) <= 1e-12 * d.energy
