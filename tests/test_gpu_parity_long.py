"""FP64 CUDA path vs the CPU oracle over the workloads' own horizons.

* The 32 x 33 x 32 Poiseuille box (Re_c 2000, dt 1e-3, seeded low-mode
  perturbation of 1e-3) for 200 steps under the reference's constant mean
  pressure gradient (re_p = 2 / Re_c, the forcing of poiseuilleflow.f90:1787).
* The 128 x 129 x 128 Re_tau 180 channel for 50 steps, with the energy
  history compared step by step.
* 400 steps on a mixed-radix box: the GPU forms the explicit terms B c of
  get_coef_rhs / get_rhs_omegay (poiseuilleflow.f90:3385-3489) as Gauss-
  Lobatto values of a derivative series; the oracle forms them as the dense
  operator products of the reference.  Both must stay within the 1e-10 bar.
* dt = 5e-4 on the 128 x 129 x 128 channel: the reference algorithm is
  unstable there from the 10% perturbation.  The oracle and the GPU path
  blow up at the same step, with the same energies up to it.

Bar: per-array relative L2 of 1e-10 on the prognostic arrays (the bar the
FP64 path must meet against the reference algorithm), 1e-7 on the (0,0)
plane averages and the Nyquist slots (parity.py).
"""
import numpy as np
import pytest

from channel_flow_gb300 import Channel, config, fields
from parity import check

pytestmark = pytest.mark.gpu


def energy(st, nny):
    """0.5 sum u^2 + v^2 + w^2 over the spectral arrays without the spanwise
    Nyquist slot: the energy print of poiseuilleflow.f90:2322-2336."""
    nyq = nny // 2
    return 0.5 * sum(float((np.delete(st[k], nyq, axis=1) ** 2).sum()) for k in ("unp1", "vnp1", "wnp1"))


def start_pair(cfg, oracle_mod, st):
    o = oracle_mod.Oracle.from_config(cfg)
    o.setup()
    o.set_state(st)
    g = Channel(cfg)
    g.upload_state(st)
    # the reference's start-up: getnonlinear in initial(), then a solve-only step
    o.getnonlinear(); o.solve()
    g.getnonlinear(); g.solve()
    return o, g


def test_c1_poiseuille_200_steps(chflow_lib, oracle_mod):
    cfg = config.CONFIGS["c1_poiseuille_32"]
    st = fields.lowmode_state(cfg, seed=1, amp=1e-3)
    o, g = start_pair(cfg, oracle_mod, st)
    with g:
        o.step(200)
        g.step(200)
        check(g.download_state(), o.get_state(), 1e-10, 1e-7)


def test_recurrence_explicit_terms_400_steps(chflow_lib, oracle_mod):
    cfg = config.small(nnx=24, nny=12, nnz=20, aphi=1.5, beta=0.75, dt=5e-4, re=300.0, re_p=1.0)
    st = fields.turbulent_start_state(cfg, seed=3)
    o, g = start_pair(cfg, oracle_mod, st)
    with g:
        o.step(400)
        g.step(400)
        check(g.download_state(), o.get_state(), 1e-10, 1e-7)


def test_c3_retau180_50_steps_energy_history(chflow_lib, oracle_mod):
    cfg = config.CONFIGS["c3_retau180_128"]
    st = fields.turbulent_start_state(cfg, seed=1)
    o, g = start_pair(cfg, oracle_mod, st)
    eo, eg = [], []
    with g:
        for _ in range(50):
            o.step(1)
            g.step(1)
            eo.append(energy({k: o.field(k) for k in ("unp1", "vnp1", "wnp1")}, cfg.nny))
            eg.append(g.diagnostics()["energy"])
        check(g.download_state(), o.get_state(), 1e-10, 1e-6)
    eo, eg = np.array(eo), np.array(eg)
    assert np.max(np.abs(eg - eo) / eo) < 1e-13, np.max(np.abs(eg - eo) / eo)


def test_c3_dt5e4_diverges_at_the_same_step(chflow_lib, oracle_mod):
    """dt = 5e-4 at 128 x 129 x 128: both the reference algorithm and the GPU
    path grow without bound from the 10% perturbation, at the same step and
    with the same energy history; the workload therefore runs at the
    reference's own dt = 2e-4 (paraandcons.f90:23)."""
    base = config.CONFIGS["c3_retau180_128"]
    cfg = config.ChannelConfig(base.nnx, base.nny, base.nnz, base.aphi, base.beta, 5e-4, base.re, base.re_p)
    st = fields.turbulent_start_state(cfg, seed=0)
    o, g = start_pair(cfg, oracle_mod, st)
    e0 = energy(st, cfg.nny)
    eo, eg = [], []
    with g:
        for _ in range(80):
            o.step(1)
            g.step(1)
            eo.append(energy({k: o.field(k) for k in ("unp1", "vnp1", "wnp1")}, cfg.nny))
            eg.append(g.diagnostics()["energy"] if np.isfinite(eo[-1]) else np.nan)
            if not np.isfinite(eo[-1]) or eo[-1] > 1e6 * e0:
                break
    eo, eg = np.array(eo), np.array(eg)
    blow = lambda e: int(np.argmax(~np.isfinite(e) | (e > 1e3 * e0)))
    assert (eo > 1e3 * e0).any() or not np.isfinite(eo).all(), "the oracle did not diverge at dt = 5e-4"
    assert blow(eo) == blow(eg), (blow(eo), blow(eg))
    n = blow(eo)
    # identical histories while the energy is still within 10x of the start
    calm = np.isfinite(eo) & (eo < 10 * e0)
    calm[n:] = False
    assert calm.sum() >= 10
    rel = np.abs(eg[calm] - eo[calm]) / eo[calm]
    assert rel.max() < 1e-10, rel.max()


def test_c4_time_step_bounded_at_5e5_not_1e4(chflow_lib):
    """The 384 x 193 x 384 Re_tau 550 channel from its wall-law start: at
    dt = 1e-4 the step (mixed path, whose nonlinear term carries the
    instability the FP64 path shows too) grows without bound within 200
    steps, at dt = 5e-5 the energy stays within 1% over 200 steps; the
    workload runs at 5e-5."""
    import bench
    base = config.CONFIGS["c4_retau550_384"]
    out = {}
    for dt in (1e-4, 5e-5):
        cfg = config.ChannelConfig(base.nnx, base.nny, base.nnz, base.aphi, base.beta, dt, base.re, base.re_p)
        st = bench.start_state(cfg, seed=0)
        with Channel(cfg, precision="mixed", zpad=300) as g:
            g.upload_state(st)
            g.getnonlinear()
            g.solve()
            e0 = g.diagnostics()["energy"]
            hist = []
            for _ in range(10):
                g.step(20)
                d = g.diagnostics()
                hist.append(d["energy"] / e0 if d["finite"] else np.inf)
                if not np.isfinite(hist[-1]):
                    break
        out[dt] = np.array(hist)
    assert (out[1e-4] > 1e6).any(), out[1e-4]
    assert np.all(np.abs(out[5e-5] - 1.0) < 0.01), out[5e-5]
