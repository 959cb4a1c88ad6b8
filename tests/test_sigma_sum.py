"""CPU check of the compensated sum of the mixed increment solve
(channel_flow_gb300/csrc/k_solve_mixed.cu, k_inc_solve): the FP32 products of
the high parts summed into S, which starts at a power of two sigma >= 8 sum|p|,
the exact remainder fma(mh, ch, S - s) plus the cross products into C, and
delta = (S - sigma) + C.  FP32 arithmetic is emulated in numpy (products of two
FP32 values are exact in FP64; the FMA is rounded once to FP32 from FP64)."""
import numpy as np

f32 = np.float32


def split(x):
    """x as hi + lo: hi its leading 24 bits, lo the next 24 (as k_inc_solve)."""
    hi = f32(x)
    lo = f32(x - np.float64(hi))
    return hi, lo


def fma32(a, b, c):
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def sigma_dot(m, c):
    """sum_k m_k c_k by the offset scheme; returns (delta, S values seen, sigma)."""
    mh, ml = zip(*(split(x) for x in m))
    ch, cl = zip(*(split(x) for x in c))
    er = np.frexp(np.sum(np.abs(np.float64(mh))))[1]   # sum |mh| < 2^er
    ec = np.frexp(np.max(np.abs(np.float64(ch))))[1]   # max |ch| < 2^ec
    sigma = f32(np.ldexp(1.0, er + ec + 3))
    S, C = sigma, f32(0.0)
    seen = []
    for k in range(len(m)):
        p = f32(np.float64(mh[k]) * np.float64(ch[k]))
        s = f32(np.float64(S) + np.float64(p))
        u = fma32(mh[k], ch[k], f32(np.float64(S) - np.float64(s)))  # S - s is exact
        S = s
        seen.append(S)
        C = f32(np.float64(C) + np.float64(u))
        C = fma32(mh[k], cl[k], C)
        C = fma32(ml[k], ch[k], C)
    # sigma is S's power of two, rounded up from a significand of 1.5 or more
    bits = np.array([S], dtype=np.float32).view(np.uint32)[0]
    sig_back = np.array([(int(bits) + 0x400000) & 0xFF800000], dtype=np.uint32).view(np.float32)[0]
    assert sig_back == sigma
    delta = np.float64(f32(np.float64(S) - np.float64(sigma))) + np.float64(C)
    return delta, np.array(seen, dtype=np.float64), float(sigma)


def test_sigma_sum_range_and_accuracy():
    rng = np.random.default_rng(3)
    worst = 0.0
    for trial in range(200):
        n = int(rng.integers(16, 66))
        m = rng.standard_normal(n) * np.exp(rng.uniform(-3, 3, n))
        c = rng.standard_normal(n) * np.exp(-0.1 * np.arange(n)) * 10.0 ** rng.uniform(-3, 3)
        delta, seen, sigma = sigma_dot(m, c)
        # S stays within (7/8, 9/8) sigma, so every S - s is exact (Sterbenz)
        assert np.all(seen > 0.875 * sigma) and np.all(seen < 1.125 * sigma)
        exact = float(np.sum(np.float64(m) * np.float64(c)))
        bound = float(np.sum(np.abs(m)) * np.max(np.abs(c)))
        worst = max(worst, abs(delta - exact) / bound)
    # about 2^-38 of sum|M| max|c| (2^-38.3 in this sample); plain FP32
    # accumulation would be ~2^-24
    assert worst < 2.0 ** -37
