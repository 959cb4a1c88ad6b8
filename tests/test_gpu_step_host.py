"""chf_step_host: advancing host-resident module arrays in place, with the
copies overlapped with the steps, gives bit for bit what
chf_upload_state + chf_step + chf_download_state give on the same arrays,
for both paths, one and several steps, and a second call continues from
the first.  Missing arrays and nsteps < 1 are rejected before any copy."""
import numpy as np
import pytest

from channel_flow_gb300 import Channel, ChannelError, config, fields
from channel_flow_gb300.fields import FIELD_NAMES, MEAN_NAMES

pytestmark = pytest.mark.gpu

CFG = config.CONFIGS["c1_poiseuille_32"]


def start():
    st = fields.reference_like_state(CFG, seed=7, epsilon=0.3, noise=0.02, gamma=5.0)
    with Channel(CFG) as g:  # a state with nonzero nonlinear histories
        g.upload_state(st)
        g.getnonlinear()
        g.solve()
        return g.download_state()


def copy(st):
    return {k: np.ascontiguousarray(st[k], dtype=np.float64).copy() for k in FIELD_NAMES + MEAN_NAMES}


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_fp64solve"])
@pytest.mark.parametrize("nsteps", [1, 3])
def test_step_host_matches_upload_step_download(chflow_lib, precision, nsteps):
    st = start()
    with Channel(CFG, precision=precision) as a:
        a.upload_state(st)
        a.step(nsteps)
        want = a.download_state()
    host = copy(st)
    with Channel(CFG, precision=precision) as b:
        b.step_host(host, nsteps)
        # a second call continues from the first, like a second chf_step
        b.step_host(host, 1)
        again = b.download_state()
    with Channel(CFG, precision=precision) as a:
        a.upload_state(st)
        a.step(nsteps)
        a.step(1)
        want2 = a.download_state()
    for k in FIELD_NAMES + MEAN_NAMES:
        assert np.array_equal(again[k], want2[k]), k
        assert np.array_equal(host[k], want2[k]), k
    host1 = copy(st)
    with Channel(CFG, precision=precision) as b:
        b.step_host(host1, nsteps)
    for k in FIELD_NAMES + MEAN_NAMES:
        assert np.array_equal(host1[k], want[k]), k


def test_step_host_rejects_bad_calls(chflow_lib):
    host = copy(start())
    with Channel(CFG, precision="mixed") as b:
        bad = dict(host)
        del bad["rhsvn"]
        with pytest.raises(ChannelError):
            b.step_host(bad, 1)
        with pytest.raises(ChannelError):
            b.step_host(host, 0)
        before = {k: v.copy() for k, v in host.items()}
        b.step_host(host, 1)  # still usable after the rejected calls
        assert any(not np.array_equal(before[k], host[k]) for k in ("vnp1", "unp1"))
