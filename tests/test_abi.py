"""C-ABI checks that need no GPU: the library builds, loads, exports every
entry point declared in include/chflow.h, and rejects bad configurations
before touching CUDA."""
import ctypes
import os
import re

import pytest

from channel_flow_gb300 import ChannelError, config
from channel_flow_gb300.channel import EXPORTS, CConfig, make_cconfig

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "chflow.h")).read()
    return sorted(set(re.findall(r"\b(chf_[a-z_0-9]+)\s*\(", src)))


def test_header_declares_exports():
    assert declared_symbols() == sorted(EXPORTS)


def test_library_exports_all_symbols(chflow_lib):
    for name in declared_symbols():
        assert hasattr(chflow_lib, name), name


def _create(lib, c):
    h = ctypes.c_void_p()
    rc = lib.chf_create(ctypes.byref(c), ctypes.byref(h))
    return rc, h, lib.chf_last_error(None).decode()


@pytest.mark.parametrize("field,value,msg", [
    ("nnx", 30, "nnx"), ("nny", 6, "nny"), ("nnz", 33, "nnz"), ("nnz", 2, "nnz"), ("nnz", 256, "nnz"),
    ("dt", 0.0, "dt"), ("re", -1.0, "re"), ("aphi", 0.0, "aphi"), ("precision", 7, "precision"),
    ("zpad", 20, "zpad"), ("nnx", 28, "nnx"),
])
def test_invalid_configs_rejected(chflow_lib, field, value, msg):
    c = make_cconfig(config.small(nnx=16, nny=8, nnz=16))
    setattr(c, field, value)
    rc, h, err = _create(chflow_lib, c)
    assert rc == -1
    assert not h.value
    assert msg in err


def test_null_handle_calls_fail_cleanly(chflow_lib):
    assert chflow_lib.chf_step(None, 1) == -1
    assert chflow_lib.chf_solve(None) == -1
    assert chflow_lib.chf_getnonlinear(None) == -1
    assert chflow_lib.chf_destroy(None) == -1
    assert chflow_lib.chf_synchronize(None) == -1


def test_transform_length_rule(chflow_lib):
    # 3*nnx/2 = 21 is not a 2,3,5-smooth length
    c = make_cconfig(config.small(nnx=16, nny=8, nnz=16))
    c.nnx = 14 * 2  # 28 -> 42 = 2*3*7
    rc, h, err = _create(chflow_lib, c)
    assert rc == -1 and "nnx" in err


def test_python_layer_raises_channel_error(chflow_lib):
    from conftest import gpu_available
    if gpu_available():
        pytest.skip("exercises the no-device path")
    from channel_flow_gb300 import Channel
    with pytest.raises(ChannelError):
        Channel(config.small(nnx=16, nny=8, nnz=16))


@pytest.mark.parametrize("nnx,nny,nnz", [(16, 8, 1025), (18, 8, 16), (16, 10, 16), (15, 8, 16),
                                          (16, 8, 15), (16, 8, 2), (0, 8, 16)])
def test_static_diagnostics_rejects_bad_grids(chflow_lib, nnx, nny, nnz):
    """The allocation-free entry point checks the plane count against its
    fixed scratch, and the grid against chf_create's rules (its layout needs
    nnx, nny multiples of 4), before touching the GPU."""
    from channel_flow_gb300.channel import CDiag
    d = CDiag()
    one = ctypes.c_void_p(16)  # never dereferenced: the size checks come first
    rc = chflow_lib.chf_diagnostics_static(nnx, nny, nnz, one, one, one, one, one, one, None,
                                           ctypes.byref(d), None)
    assert rc == -1


def test_batch_rejects_mixed_devices_and_bad_channels(chflow_lib):
    base = make_cconfig(config.CONFIGS["c1_poiseuille_32"])
    other = make_cconfig(config.CONFIGS["c1_poiseuille_32"], device=1)
    arr = (CConfig * 2)(base, other)
    b = ctypes.c_void_p()
    assert chflow_lib.chf_batch_create(2, arr, ctypes.byref(b)) == -1
    assert "one device" in chflow_lib.chf_batch_last_error(None).decode()
    bad = make_cconfig(config.CONFIGS["c1_poiseuille_32"])
    bad.nnz = 33
    arr = (CConfig * 2)(base, bad)
    rc = chflow_lib.chf_batch_create(2, arr, ctypes.byref(b))
    assert rc != 0 and not b.value
    assert chflow_lib.chf_batch_create(0, arr, ctypes.byref(b)) == -1
    assert chflow_lib.chf_batch_step(None, 1) == -1
    assert chflow_lib.chf_batch_destroy(None) == -1
    assert chflow_lib.chf_write_restart(None, b".", 1, 2, -1) == -1
    assert chflow_lib.chf_read_restart(None, b".", 1, 2, -1) == -1
