"""The autotuner (chf_autotune), through the C ABI: it leaves the state as it
found it, the tuned step still matches the oracle, and later handles of the
same grid start from the cached choice."""
import numpy as np
import pytest

from channel_flow_gb300 import Channel, ChannelError, config, fields
from channel_flow_gb300.fields import FIELD_NAMES, MEAN_NAMES
from parity import check

pytestmark = pytest.mark.gpu

# a grid on the shared-memory FFT path (36- and 18-point x / y lines, 40- and 72-point
# z lines), so every knob has candidates
CFG = config.small(nnx=24, nny=12, nnz=20, aphi=1.5, beta=0.75, dt=5e-4, re=300.0, re_p=1.0)


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_fp64solve"])
def test_autotune_keeps_state_and_caches(chflow_lib, precision):
    st = fields.turbulent_start_state(CFG, seed=12)
    with Channel(CFG, precision=precision, zpad=36) as g:
        assert "not tuned" in g.tuning()
        g.upload_state(st)
        g.getnonlinear()
        g.solve()
        before = g.download_state()
        report = g.autotune(reps=2)
        after = g.download_state()
        assert "rules" in report and "not tuned" not in report, report
        for k in FIELD_NAMES + MEAN_NAMES:
            assert np.array_equal(before[k], after[k]), k
    with Channel(CFG, precision=precision, zpad=36) as h:
        assert h.tuning() == report


def test_tuned_step_matches_oracle(chflow_lib, oracle_mod):
    st = fields.reference_like_state(CFG, seed=4, epsilon=0.3, noise=0.02, gamma=5.0)
    o = oracle_mod.Oracle.from_config(CFG)
    o.setup()
    o.set_state(st)
    o.getnonlinear(); o.solve(); o.step(10)
    with Channel(CFG, precision="fp64") as g:
        g.upload_state(st)
        g.autotune(reps=1)
        g.getnonlinear(); g.solve(); g.step(10)
        check(g.download_state(), o.get_state(), 1e-10, 1e-7)


def test_autotune_needs_a_state(chflow_lib):
    with Channel(CFG) as g:
        with pytest.raises(ChannelError) as ei:
            g.autotune()
        assert ei.value.code == -4
