"""The allocation-free entry point chf_diagnostics_static, through the C ABI.

It exists for callers that cannot allocate device memory: a host model whose
device memory belongs to another runtime's pool, a run that has committed
the device's memory to the resident state, or a time loop that must not pay
for cudaMalloc/cudaFree.  Its results must agree with chf_diagnostics, the
entry point that reduces into handle-owned scratch, on the same device
arrays, on two calls in a row.  The shared static scratch keeps the last
call's values, so the calls go from a larger grid to a smaller one: a stale
plane of the larger grid would show in the smaller grid's results.  Each
plane's energy is also checked against NumPy on the downloaded fields.
This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

from channel_flow_gb300 import Channel, config, fields
from channel_flow_gb300.channel import CDiag

pytestmark = pytest.mark.gpu

# larger grid first (more wall-normal planes), then a smaller one
GRIDS = [
    config.small(nnx=24, nny=12, nnz=40, aphi=1.5, beta=0.75, dt=5e-4, re=300.0, re_p=1.0),
    config.small(nnx=16, nny=8, nnz=16, aphi=1.0, beta=0.5, dt=5e-4, re=180.0, re_p=1.0),
]


def _dev(ch, which):
    p = ctypes.c_void_p()
    assert ch.L.chf_device_field(ch.h, which, ctypes.byref(p)) == 0
    return p


def _plane_energy(state, cfg):
    """0.5 sum (u^2 + v^2 + w^2) per wall-normal plane, spanwise Nyquist row
    excluded, on the downloaded spectral arrays."""
    nyq = cfg.nny // 2
    e = np.zeros(cfg.nnz + 1)
    for k in ("unp1", "vnp1", "wnp1"):
        a = np.delete(state[k], nyq, axis=1)
        e += 0.5 * (a ** 2).sum(axis=(1, 2))
    return e


def test_static_diagnostics_match_handle_diagnostics(chflow_lib):
    for seed, cfg in enumerate(GRIDS):
        st = fields.reference_like_state(cfg, seed=seed, epsilon=0.3, noise=0.02, gamma=5.0)
        with Channel(cfg) as ch:
            ch.upload_state(st)
            ch.getnonlinear()
            ch.solve()
            ch.synchronize()
            ref = ch.diagnostics()
            planes = _plane_energy(ch.download_state(), cfg)
            # field slots: 0 vnp1, 1 omegaynp1, 2 unp1, 3 wnp1, 4 omegaxnp1, 5 omegaznp1
            ptrs = [_dev(ch, i) for i in (2, 0, 3, 4, 1, 5)]
            for call in range(2):
                prof = np.full(cfg.nnz + 1, np.nan)
                d = CDiag()
                rc = chflow_lib.chf_diagnostics_static(
                    cfg.nnx, cfg.nny, cfg.nnz, *ptrs,
                    prof.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(d), None)
                assert rc == 0, (cfg, call)
                assert d.finite == 1
                assert abs(d.energy - ref["energy"]) <= 1e-12 * ref["energy"], (cfg, call)
                assert d.max_abs == ref["max_abs"], (cfg, call)
                assert np.allclose(prof, planes, rtol=1e-12, atol=1e-14 * planes.max()), (cfg, call)
                assert abs(prof.sum() - d.energy) <= 1e-12 * d.energy
