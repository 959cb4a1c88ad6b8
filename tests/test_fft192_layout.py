"""CPU check of the register FFT's factorisation and lane tables
(channel_flow_gb300/csrc/fft_warp.cuh): 192 = 6 x 32, a 6-point DFT per lane,
a twiddle W192^(lane k1), and five cross-lane radix-2 stages in which every
lane computes y = p + S v and multiplies by W' (S = -1 and W' = the stage
twiddle on the upper lane of a butterfly, S = +1 and W' = 1 on the lower one),
emulated per lane in numpy against numpy's FFT."""
import numpy as np
import pytest

TW = np.exp(-2j * np.pi * np.arange(192) / 192)


def twid(m, sign):
    w = TW[m % 192]
    return np.conj(w) if sign > 0 else w


def tables(sign):
    """Stage twiddles W' and signs S per (stage, lane), and W192^(lane k1)."""
    st = np.ones((5, 32), complex)
    sg = np.ones((5, 32))
    for s in range(5):
        h = 16 >> s
        for lane in range(32):
            if lane & h:
                st[s, lane] = twid((lane & (h - 1)) * (96 // h), sign)
                sg[s, lane] = -1.0
    t6 = np.array([[twid(lane * k1, sign) for lane in range(32)] for k1 in range(6)])
    return st, sg, t6


def dft6(a, sign):
    j = np.arange(6)
    return np.exp(sign * 2j * np.pi * np.outer(j, j) / 6) @ a


def shfl_xor(a, h):
    return a[:, np.arange(32) ^ h]


def natural_to_perm(a, sign):
    st, sg, t6 = tables(sign)
    a = dft6(a, sign) * t6
    for s in range(5):
        a = (sg[s] * a + shfl_xor(a, 16 >> s)) * st[s]
    return a


def perm_to_natural(a, sign):
    st, sg, t6 = tables(sign)
    for s in (4, 3, 2, 1, 0):
        x = a * st[s]
        a = sg[s] * x + shfl_xor(x, 16 >> s)
    return dft6(a * t6, sign)


def bitrev5(x):
    return int(f"{x:05b}"[::-1], 2)


@pytest.mark.parametrize("sign", [+1, -1])
def test_fft192_lane_layouts(sign):
    rng = np.random.default_rng(4)
    x = rng.standard_normal(192) + 1j * rng.standard_normal(192)
    X = np.fft.fft(x) if sign < 0 else np.fft.ifft(x) * 192
    natural = lambda v: np.array([[v[32 * j + lane] for lane in range(32)] for j in range(6)])
    permuted = lambda v: np.array([[v[k1 + 6 * bitrev5(lane)] for lane in range(32)] for k1 in range(6)])
    # natural input -> value k1 of lane l holds element k1 + 6 bitrev5(l)
    assert np.abs(natural_to_perm(natural(x), sign) - permuted(X)).max() < 1e-12
    # permuted input -> natural output
    assert np.abs(perm_to_natural(permuted(x), sign) - natural(X)).max() < 1e-12
