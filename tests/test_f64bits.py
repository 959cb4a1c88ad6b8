"""The integer-operation FP64 <-> FP32 helpers used by the mixed path's
kernels (channel_flow_gb300/csrc/f64bits.cuh), compiled as host code and
checked against the compiler's IEEE conversions: narrowing rounds to
nearest, splitting gives the leading 24 bits plus the next 23, widening is
exact, binary32 subnormals flush to zero."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_f64bits_host(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "f64bits_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-o", exe, os.path.join(HERE, "f64bits_check.cpp")], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip() == "ok"
