"""chf_statistics against the reference's physical-space statistics."""
import numpy as np
import pytest

from channel_flow_gb300 import Channel, config, fields
from stats_ref import statistics

pytestmark = pytest.mark.gpu

CASES = [config.CONFIGS["c1_poiseuille_32"],
         config.small(nnx=24, nny=12, nnz=20, aphi=1.5, beta=0.75, dt=5e-4, re=300.0, re_p=1.0)]


@pytest.mark.parametrize("cfg", CASES)
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_statistics_match_physical_space(chflow_lib, cfg, precision):
    st = fields.turbulent_start_state(cfg, seed=4)
    with Channel(cfg, precision=precision) as g:
        g.upload_state(st)
        g.getnonlinear(); g.solve(); g.step(10)
        got = g.statistics()
        state = g.download_state()
    ref = statistics(cfg, state)
    scale = {"u": np.abs(ref["u"]).max()}
    for k in ("u", "v", "w"):
        assert np.allclose(got[k], ref[k], rtol=0, atol=1e-12 * scale["u"]), k
    cov = max(np.abs(ref[k]).max() for k in ("uu", "vv", "ww"))
    for k in ("uu", "vv", "ww", "uv", "uw", "vw"):
        assert np.allclose(got[k], ref[k], rtol=0, atol=1e-11 * cov), k
    assert np.allclose(got["z"], ref["z"], atol=1e-15)
    for k in ("energy", "u_tau_top", "u_tau_bottom", "re_centre", "re_bulk"):
        assert abs(got[k] - ref[k]) <= 1e-10 * abs(ref[k]), (k, got[k], ref[k])
    assert abs(got["re_tau_top"] - got["u_tau_top"] * cfg.re) < 1e-12 * got["re_tau_top"]
    assert abs(got["bulk_velocity"] - fields.bulk_velocity(state)) < 1e-14


def test_laminar_statistics(chflow_lib):
    """U = 1 - z^2: u_tau^2 = 2 / re at both walls, Re_c = re, U_b = 2/3, no fluctuations."""
    cfg = CASES[0]
    with Channel(cfg) as g:
        g.upload_state(fields.laminar_state(cfg))
        s = g.statistics()
    assert abs(s["u_tau_top"] ** 2 - 2.0 / cfg.re) < 1e-14
    assert abs(s["u_tau_bottom"] ** 2 - 2.0 / cfg.re) < 1e-14
    assert abs(s["re_centre"] - cfg.re) < 1e-10
    assert abs(s["bulk_velocity"] - 2.0 / 3.0) < 1e-15
    assert np.abs(s["uu"]).max() == 0.0 and np.abs(s["uv"]).max() == 0.0
