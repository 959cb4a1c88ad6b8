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


# every launch shape of the increment solve: (modes per CTA, columns per load
# batch, rows per thread)
INC_SHAPES = [(4, 3, 1), (4, 2, 1), (4, 4, 1), (2, 2, 1), (2, 3, 1), (2, 4, 1),
              (4, 2, 2), (4, 3, 2), (2, 2, 2), (2, 3, 2)]


def test_increment_solve_shapes_bit_identical(chflow_lib):
    # the k^2 groups of this grid hold 1 to 7 modes, so groups span several
    # CTAs at either modes-per-CTA setting
    st = fields.turbulent_start_state(CFG, seed=3)
    ref = None
    for m, c, r in INC_SHAPES:
        with Channel(CFG, precision="mixed", zpad=36) as g:
            g.set_launch_shape("inc_rows", 1)  # the handle may start from a cached choice
            g.set_launch_shape("inc_modes", m)
            g.set_launch_shape("inc_columns", c)
            g.set_launch_shape("inc_rows", r)
            assert "set by chf_set_launch_shape" in g.tuning()
            assert f"increment solve {m} modes x {c} columns x {r} rows per thread" in g.tuning()
            g.upload_state(st)
            g.getnonlinear()
            g.solve()
            g.step(4)
            out = g.download_state()
        if ref is None:
            ref = out
            continue
        for k in FIELD_NAMES + MEAN_NAMES:
            assert np.array_equal(ref[k], out[k]), ((m, c, r), k)


def test_increment_solve_wide_blocks_bit_identical(chflow_lib):
    # 2 (nnz + 1) = 322 block rows: one pass of 352 threads, or 288-thread blocks that loop
    cfg = config.small(nnx=8, nny=8, nnz=160, aphi=1.0, beta=0.5, dt=2e-4, re=180.0, re_p=1.0)
    st = fields.turbulent_start_state(cfg, seed=5)
    outs = []
    for wide in (1, 0):
        with Channel(cfg, precision="mixed") as g:
            g.set_launch_shape("inc_rows", 1)
            g.set_launch_shape("inc_wide", wide)
            g.upload_state(st)
            g.getnonlinear()
            g.solve()
            g.step(3)
            outs.append(g.download_state())
    for k in FIELD_NAMES + MEAN_NAMES:
        assert np.array_equal(outs[0][k], outs[1][k]), k


def test_set_launch_shape_rejects(chflow_lib):
    with Channel(CFG, precision="mixed", zpad=36) as g:
        before = g.tuning()
        for name, value in [("inc_modes", 3), ("inc_columns", 5), ("inc_rows", 3), ("kxb", 7),
                            ("no_such_shape", 1)]:
            with pytest.raises(ChannelError) as ei:
                g.set_launch_shape(name, value)
            assert ei.value.code == -1, (name, value)
        g.set_launch_shape("inc_rows", 1)
        g.set_launch_shape("inc_columns", 4)
        with pytest.raises(ChannelError):
            g.set_launch_shape("inc_rows", 2)  # two rows per thread take 2 or 3 columns
        assert "4 columns x 1 rows per thread" in g.tuning()
        assert "set by chf_set_launch_shape" in g.tuning() and before != g.tuning()
