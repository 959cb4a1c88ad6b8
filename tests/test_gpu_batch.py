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


def class_cfgs():
    """Two classes of stacked channels (identical grids, uneven Reynolds
    numbers) in both mixed forms, plus an FP64 channel and a lone grid."""
    base = dict(aphi=1.0, beta=0.5, dt=5e-4, re_p=1.0)
    out, precs = [], []
    for re in (150.0, 180.0, 220.0, 260.0, 300.0):
        out.append(config.small(nnx=16, nny=8, nnz=16, re=re, **base))
        precs.append("mixed_fp64solve")
    for re in (200.0, 240.0, 280.0):
        out.append(config.small(nnx=24, nny=12, nnz=20, re=re, aphi=1.5, beta=0.75, dt=5e-4, re_p=1.0))
        precs.append("mixed")
    out.append(config.small(nnx=16, nny=8, nnz=16, re=190.0, **base))
    precs.append("fp64")
    out.append(config.small(nnx=32, nny=16, nnz=24, re=210.0, **base))
    precs.append("mixed_fp64solve")
    return out, precs


def test_stacked_classes_match_single_channels(chflow_lib):
    cfgs, precs = class_cfgs()
    sts = [fields.turbulent_start_state(c, seed=20 + i) for i, c in enumerate(cfgs)]
    def bulk(st):  # (1/2) int u dz of the (0,0) mode, from au0
        a = st["au0"][:, 0]
        return sum(a[n] / (1.0 - n * n) for n in range(0, len(a), 2))

    # constant flow rate on one member of each class
    flow = {1: 1.01 * bulk(sts[1]), 6: 0.99 * bulk(sts[6])}
    with Batch(cfgs, precision=precs) as b:
        for i, (ch, st) in enumerate(zip(b, sts)):
            ch.upload_state(st)
            if i in flow:
                ch.set_flow_rate(flow[i])
            ch.getnonlinear()
            ch.solve()
        b.step(5)
        b.step(4)
        b.synchronize()
        got = [ch.download_state() for ch in b]
        rates = [ch.flow_rate() for ch in b]
    for i, (cfg, prec, st, g) in enumerate(zip(cfgs, precs, sts, got)):
        with Channel(cfg, precision=prec) as c:
            c.upload_state(st)
            if i in flow:
                c.set_flow_rate(flow[i])
            c.getnonlinear()
            c.solve()
            c.step(9)
            ref = c.download_state()
            assert c.flow_rate() == rates[i], i
        for k in FIELD_NAMES + MEAN_NAMES:
            assert np.array_equal(g[k], ref[k]), (i, prec, k)
