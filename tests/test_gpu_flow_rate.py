"""Constant flow rate (chf_set_flow_rate): the bulk velocity stays at its
target while the mean pressure gradient adjusts; on the laminar fixed point
the control is idle and the run equals the constant-pressure run."""
import numpy as np
import pytest

from channel_flow_gb300 import Channel, config, fields

pytestmark = pytest.mark.gpu

CFG = config.CONFIGS["c1_poiseuille_32"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_bulk_velocity_is_held(chflow_lib, precision):
    st = fields.lowmode_state(CFG, seed=11, amp=1e-3)
    ub0 = fields.bulk_velocity(st)
    with Channel(CFG, precision=precision) as g:
        g.set_flow_rate(ub0)
        g.upload_state(st)
        g.getnonlinear(); g.solve(); g.step(200)
        out = g.download_state()
        fr = g.flow_rate()
    ub = fields.bulk_velocity(out)
    assert abs(ub - ub0) < 1e-12 * ub0, (ub, ub0)
    assert abs(fr["bulk_velocity"] - ub0) < 1e-12 * ub0
    assert fr["target"] == ub0


def test_pressure_gradient_responds(chflow_lib):
    """A 10% faster target needs an extra driving gradient, a slower one a
    braking one; without control the bulk velocity of the laminar flow stays."""
    st = fields.laminar_state(CFG)
    ub0 = fields.bulk_velocity(st)
    assert abs(ub0 - 2.0 / 3.0) < 1e-14
    res = {}
    for f in (1.1, 0.9):
        with Channel(CFG) as g:
            g.set_flow_rate(f * ub0)
            g.upload_state(st)
            g.getnonlinear(); g.solve(); g.step(20)
            res[f] = g.flow_rate()
            assert abs(fields.bulk_velocity(g.download_state()) - f * ub0) < 1e-12
    assert res[1.1]["dpdx_correction"] > 0 > res[0.9]["dpdx_correction"]


def test_idle_on_the_laminar_fixed_point(chflow_lib):
    st = fields.laminar_state(CFG)
    outs = []
    for control in (False, True):
        with Channel(CFG) as g:
            if control:
                g.set_flow_rate(fields.bulk_velocity(st))
            g.upload_state(st)
            g.getnonlinear(); g.solve(); g.step(50)
            outs.append(g.download_state())
            if control:
                assert abs(g.flow_rate()["dpdx_correction"]) < 1e-12
    for k in ("vnp1", "unp1", "au0"):
        assert np.allclose(outs[0][k], outs[1][k], rtol=0, atol=1e-13), k


def test_flow_rate_rejects_bad_values(chflow_lib):
    with Channel(CFG) as g:
        for bad in (-1.0, float("nan"), float("inf")):
            with pytest.raises(Exception, match="bulk velocity"):
                g.set_flow_rate(bad)
        g.set_flow_rate(0.0)
        assert g.flow_rate()["target"] == 0.0
