"""CPU checks of the fixed-point digit formats of the exact tensor-core GEMMs
(channel_flow_gb300/csrc/k_tcgemm.cu): the K limits that keep every level's
FP32 sum an exact integer, and the accuracy each format gives, by a numpy
emulation of the digit split and the level sums."""
import numpy as np
import pytest

# (planes, radix bits, K limit the launcher enforces)
FORMATS = [(4, 7, 680), (3, 8, 204)]


def digits(x, e, planes, rb):
    """planes digits of x * 2^-e: each the rint of the scaled remainder."""
    y = np.ldexp(x, rb - e)
    out = []
    for _ in range(planes):
        d = np.rint(y)
        out.append(d)
        y = (y - d) * 2.0 ** rb
    return out


def fx_gemm(a, b, planes, rb):
    """C = A B from per-row / per-column digit planes and exact level sums."""
    ea = np.frexp(np.abs(a).max(axis=1))[1]
    eb = np.frexp(np.abs(b).max(axis=0))[1]
    ad = digits(a, ea[:, None], planes, rb)
    bd = digits(b, eb[None, :], planes, rb)
    acc = np.zeros((a.shape[0], b.shape[1]))
    for level in range(planes):
        s = sum(ad[i] @ bd[level - i] for i in range(level + 1))
        assert np.all(np.abs(s) < 2.0 ** 24)  # exact in FP32
        acc += s * 2.0 ** (-rb * level)
    return acc * np.ldexp(1.0, ea[:, None] + eb[None, :] - 2 * rb)


@pytest.mark.parametrize("planes,rb,kmax", FORMATS)
def test_digit_ranges_and_level_bound(planes, rb, kmax):
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, 100000)
    d = digits(x, 0, planes, rb)
    half = 2 ** (rb - 1)
    assert np.abs(d[0]).max() <= 2 * half  # first digit: rb + 1 bits
    for di in d[1:]:
        assert np.abs(di).max() <= half
    # every digit is an integer of at most 9 bits: exact in bf16
    assert all(np.all(di == np.rint(di)) and np.abs(di).max() <= 256 for di in d)
    # the largest level's products per k (all digits at their bounds) times
    # the K limit stays below 2^24
    top = [2 * half] + [half] * (planes - 1)
    worst = max(sum(top[i] * top[lv - i] for i in range(lv + 1)) for lv in range(planes))
    assert worst * kmax < 2 ** 24
    assert worst * (kmax + 16) >= 2 ** 24  # the limit is within one K16 step of the bound


@pytest.mark.parametrize("planes,rb,tol", [(4, 7, 2.0 ** -27), (3, 8, 2.0 ** -23)])
def test_emulated_gemm_accuracy(planes, rb, tol):
    rng = np.random.default_rng(2)
    m, k, n = 40, 144, 64
    a = np.cos(np.pi * np.outer(np.arange(m), np.arange(k)) / 200.0)
    b = rng.standard_normal((k, n)) * np.exp(-0.05 * np.arange(k))[:, None]
    b = b.astype(np.float32).astype(np.float64)  # B data are taken as FP32
    c = fx_gemm(a, b, planes, rb)
    ref = a @ b
    scale = np.abs(a).max(axis=1)[:, None] * np.abs(b).max(axis=0)[None, :] * k
    assert np.all(np.abs(c - ref) <= tol * scale)
