"""Restart files through the CUDA library: chf_write_restart writes what
the host reader and the reference's layout expect, and a run restarted from
the files continues bit for bit like the uninterrupted run."""
import numpy as np
import pytest

from channel_flow_gb300 import Channel, config, fields, restart
from channel_flow_gb300.fields import FIELD_NAMES, MEAN_NAMES

pytestmark = pytest.mark.gpu

CFG = config.CONFIGS["c1_poiseuille_32"]


def start():
    return fields.reference_like_state(CFG, seed=4, epsilon=0.3, noise=0.02, gamma=5.0)


@pytest.mark.parametrize("nproc", [1, 4])
def test_write_matches_host_reader(chflow_lib, tmp_path, nproc):
    with Channel(CFG) as g:
        g.upload_state(start())
        g.getnonlinear()   # the reference writes after getnonlinear (output, REF:225)
        g.write_restart(str(tmp_path), nproc=nproc)
        now = g.download_state()
    back = restart.read_restart(CFG, str(tmp_path), nproc=nproc)
    for k in restart.REC1 + restart.REC2:
        assert np.array_equal(back[k], now[k]), k


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_restarted_run_continues_exactly(chflow_lib, tmp_path, precision):
    with Channel(CFG, precision=precision) as a:
        a.upload_state(start())
        a.getnonlinear(); a.solve(); a.step(3)
        a.getnonlinear()
        a.write_restart(str(tmp_path), nproc=2, istep=4)
        a.solve(); a.step(5)
        ref = a.download_state()
    with Channel(CFG, precision=precision) as b:
        b.read_restart(str(tmp_path), nproc=2, istep=4)
        b.solve(); b.step(5)   # the reference's istep = istepbegin iteration, then the loop
        got = b.download_state()
    nyq = CFG.nny // 2
    for k in FIELD_NAMES + MEAN_NAMES:
        if k in ("omegaxnp1", "omegaznp1"):
            # not in the file; the spanwise Nyquist slot of these two is never
            # written by the mixed path's solve (no step reads it)
            ref[k][:, nyq, :] = 0.0
            got[k][:, nyq, :] = 0.0
        assert np.array_equal(got[k], ref[k]), k


def test_host_written_files_load(chflow_lib, tmp_path):
    st = start()
    restart.write_restart(CFG, st, str(tmp_path), nproc=4, tag=7)
    with Channel(CFG) as g:
        g.read_restart(str(tmp_path), nproc=4, tag=7)
        back = g.download_state()
    for k in restart.REC1 + restart.REC2:
        assert np.array_equal(back[k], st[k]), k


def test_restart_errors(chflow_lib, tmp_path):
    with Channel(CFG) as g:
        with pytest.raises(Exception, match="chf_write_restart before"):
            g.write_restart(str(tmp_path))
        with pytest.raises(Exception, match="cannot open"):
            g.read_restart(str(tmp_path))
        g.upload_state(start())
        with pytest.raises(Exception, match="multiple of 2 nproc"):
            g.write_restart(str(tmp_path), nproc=3)
