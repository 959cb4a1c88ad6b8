"""Orr-Sommerfeld known answer on the GPU, FP64 and mixed: a 2D eigenmode of
amplitude 1e-6 seeded on Poiseuille flow at re = 7500 (box 2 pi x 2 pi x 2,
16 x 4 x 64, alpha = 1, dt = 1e-3), 5000 steps; the growth rate and phase
speed from the amplitude history and the growth rate from the perturbation
energy history are matched to the eigenvalue of the collocation operator, and
the FP64 path's rates to the oracle's run."""
import pytest

from channel_flow_gb300 import Channel, config, fields

from os_growth import fit_rates, run_history

CFG = config.CONFIGS["c2_orr_sommerfeld"]
NSTEPS, CHUNK, SKIP = 5000, 250, 2

# Relative tolerances on Re(sigma) (amplitude fit, energy fit) and Im(sigma).
# The FP64 bars leave room for the O(dt^2) error of the AB2/CN scheme and the
# start-up transient.  The mixed path carries the 1e-6 perturbation on an
# O(1) base flow in FP32 physical values, whose rounding (one ulp of 1 is
# 1.2e-7) is a few per cent of the perturbation at every point.
TOL = {"fp64": (1e-3, 5e-3, 1e-4), "mixed": (1e-2, 2e-2, 3e-4)}


def _gpu_history(precision, nsteps=NSTEPS):
    st = fields.orr_sommerfeld_state(CFG)
    with Channel(CFG, precision=precision) as ch:
        ch.upload_state(st)
        return run_history(ch.step, ch.download_state, st, CFG, nsteps, CHUNK)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_os_growth_rate(chflow_lib, precision):
    sigma, _ = fields.orr_sommerfeld_mode(CFG)
    t, amp, en = _gpu_history(precision)
    s, er = fit_rates(t, amp, en, SKIP)
    tre, ten, tim = TOL[precision]
    print(f"{precision}: sigma {s} energy-rate {er} eigenvalue {sigma}")
    assert abs(s.real - sigma.real) < tre * abs(sigma.real)
    assert abs(er - sigma.real) < ten * abs(sigma.real)
    assert abs(s.imag - sigma.imag) < tim * abs(sigma.imag)


@pytest.mark.gpu
def test_os_growth_matches_oracle(chflow_lib, oracle_mod):
    n = 2000
    st = fields.orr_sommerfeld_state(CFG)
    o = oracle_mod.Oracle.from_config(CFG)
    o.set_state(st)
    to, ao, eo = run_history(o.step, o.get_state, st, CFG, n, CHUNK)
    tg, ag, eg = _gpu_history("fp64", n)
    so, ero = fit_rates(to, ao, eo, SKIP)
    sg, erg = fit_rates(tg, ag, eg, SKIP)
    assert abs(sg - so) < 1e-7 * abs(so)
    assert abs(erg - ero) < 1e-6 * abs(ero)
