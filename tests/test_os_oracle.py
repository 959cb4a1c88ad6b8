"""Orr-Sommerfeld known answer on the CPU: the oracle's growth of a seeded
eigenmode (re = 7500, alpha = 1, 16 x 4 x 64, dt = 1e-3) against the
eigenvalue of the same collocation operator.  This pins the oracle's time step
to a physical known answer independent of any implementation."""
import dataclasses

import numpy as np
import pytest

from channel_flow_gb300 import config, fields

from os_growth import fit_rates, run_history

CFG = config.CONFIGS["c2_orr_sommerfeld"]


def test_eigen_solver_classical_value():
    # Orszag (J. Fluid Mech. 50, 1971): c = 0.23752649 + 0.00373967 i at
    # re = 10000, alpha = 1 for plane Poiseuille flow.
    cfg = dataclasses.replace(CFG, re=10000.0, re_p=2.0 / 10000.0)
    sigma, _ = fields.orr_sommerfeld_mode(cfg)
    c = 1j * sigma  # v ~ exp(i alpha (x - c t)), alpha = 1
    assert abs(c.real - 0.23752649) < 2e-8
    assert abs(c.imag - 0.00373967) < 2e-8


def test_eigenmode_satisfies_wall_conditions():
    sigma, vec = fields.orr_sommerfeld_mode(CFG)
    j = np.arange(CFG.nnz + 1)
    vec = vec / np.abs(vec).max()
    for row in (np.ones_like(j), (-1.0) ** j, j ** 2, -((-1.0) ** j) * j ** 2):
        assert abs(np.dot(row, vec)) < 1e-12 * np.abs(row).sum()
    assert sigma.real > 0.0  # re = 7500 lies above the critical 5772


def test_oracle_growth_rate(oracle_mod):
    sigma, _ = fields.orr_sommerfeld_mode(CFG)
    st = fields.orr_sommerfeld_state(CFG)
    o = oracle_mod.Oracle.from_config(CFG)
    o.set_state(st)
    t, amp, en = run_history(o.step, o.get_state, st, CFG, 2000, 100)
    s, er = fit_rates(t, amp, en, skip=5)
    assert abs(s.real - sigma.real) < 1e-3 * abs(sigma.real)
    assert abs(s.imag - sigma.imag) < 1e-4 * abs(sigma.imag)
    assert abs(er - sigma.real) < 5e-3 * abs(sigma.real)
