"""Failure detection of the tensor-core pipeline, without a GPU fault: the
exact GEMMs bound every mbarrier wait; chf_test_wait_timeout makes the next
GEMM launch leave its first stage without data, so its waits run out after a
few milliseconds.  The kernel must unwind (copies landed, MMAs drained,
tensor memory freed), the host must see CHF_E_CUDA with the wait's code, and
the handle must step normally afterwards."""
import numpy as np
import pytest

from channel_flow_gb300 import Channel, ChannelError, config, fields
from channel_flow_gb300.fields import FIELD_NAMES, MEAN_NAMES

pytestmark = pytest.mark.gpu

CFG = config.small(nnx=24, nny=12, nnz=20, aphi=1.5, beta=0.75, dt=5e-4, re=300.0, re_p=1.0)


@pytest.mark.parametrize("precision", ["mixed", "mixed_fp64solve"])
def test_wait_timeout_is_reported_and_recovered(chflow_lib, precision):
    st = fields.turbulent_start_state(CFG, seed=3)
    with Channel(CFG, precision=precision) as ref:
        ref.upload_state(st)
        ref.getnonlinear(); ref.solve(); ref.step(3)
        want = ref.download_state()
    with Channel(CFG, precision=precision) as g:
        g.upload_state(st)
        g.test_wait_timeout(5000)  # 5 ms
        g.getnonlinear()
        with pytest.raises(ChannelError) as ei:
            g.synchronize()
        assert ei.value.code == -2
        assert "tensor-core pipeline wait timed out" in str(ei.value)
        # reported once; the handle is usable again from a fresh state
        g.synchronize()
        g.upload_state(st)
        g.getnonlinear(); g.solve(); g.step(3)
        g.synchronize()
        got = g.download_state()
    for k in FIELD_NAMES + MEAN_NAMES:
        assert np.array_equal(got[k], want[k]), k


def test_wait_timeout_rejected_for_fp64(chflow_lib):
    with Channel(CFG, precision="fp64") as g:
        with pytest.raises(ChannelError) as ei:
            g.test_wait_timeout(5000)
        assert ei.value.code == -1
