"""Ensembles (chf_batch): channels of uneven size, Reynolds number and
precision stepped together give bit-identical results to stepping each
alone, through the graph (pairs) and the direct (odd remainder) paths."""
import numpy as np
import pytest

from channel_flow_gb300 import Batch, Channel, config, fields
from channel_flow_gb300.fields import FIELD_NAMES, MEAN_NAMES

pytestmark = pytest.mark.gpu

CFGS = [config.small(nnx=16, nny=8, nnz=16, aphi=1.0, beta=0.5, dt=5e-4, re=180.0, re_p=1.0),
        config.small(nnx=24, nny=12, nnz=20, aphi=1.5, beta=0.75, dt=5e-4, re=300.0, re_p=1.0),
        config.CONFIGS["c1_poiseuille_32"]]
PRECS = ["fp64", "mixed", "fp64"]


def states():
    return [fields.reference_like_state(c, seed=10 + i, epsilon=0.3, noise=0.02, gamma=5.0)
            for i, c in enumerate(CFGS)]


def test_batch_matches_single_channels(chflow_lib):
    sts = states()
    with Batch(CFGS, precision=PRECS) as b:
        assert len(b) == 3
        for ch, st in zip(b, sts):
            ch.upload_state(st)
            ch.getnonlinear()
            ch.solve()
        b.step(7)
        b.step(2)
        b.synchronize()
        got = [ch.download_state() for ch in b]
    for cfg, prec, st, g in zip(CFGS, PRECS, sts, got):
        with Channel(cfg, precision=prec) as c:
            c.upload_state(st)
            c.getnonlinear()
            c.solve()
            c.step(9)
            ref = c.download_state()
        for k in FIELD_NAMES + MEAN_NAMES:
            assert np.array_equal(g[k], ref[k]), (cfg, k)


def test_batch_requires_every_state(chflow_lib):
    sts = states()
    with Batch(CFGS[:2]) as b:
        b[0].upload_state(sts[0])
        with pytest.raises(Exception, match="channel 1 has no state"):
            b.step(2)
