"""chf_pressure: the total-head pressure from the Lamb vector, against a
dense NumPy collocation solve fed with the extended-precision Lamb vector,
and the laminar closed form."""
import numpy as np
import pytest

from channel_flow_gb300 import Channel, config, fields
from exact_lamb import lamb

pytestmark = pytest.mark.gpu

CASES = {
    "small16": config.small(nnx=16, nny=8, nnz=16, aphi=1.0, beta=0.5, dt=5e-4, re=180.0, re_p=1.0),
    "mixed_radix": config.small(nnx=24, nny=12, nnz=20, aphi=1.5, beta=0.75, dt=5e-4, re=300.0, re_p=1.0),
}


def pressure_ref(cfg, st):
    """Per mode: (D^2 - k^2) P = -(i a H1 + D H2 + i b H3) at z_1..z_{N-1},
    D P(+-1) = -H2 + (D^2 v - k^2 v) / re, dense solve; (0,0): P = -int H2, zero mean."""
    n = cfg.nnz
    T0, T2, _ = fields.collocation_matrices(n)
    D = fields.cheb_derivative_matrix(n)
    h1, h2, h3 = (fields.as_complex(np.ascontiguousarray(h, dtype=np.float64)) for h in lamb(cfg, st))
    v = fields.as_complex(st["vnp1"])
    ia, ib = fields.wavenumbers(cfg)
    P = np.zeros(v.shape, complex)
    j = np.arange(n + 1)
    top, bot = j ** 2.0, -((-1.0) ** j) * j ** 2.0
    for ky in range(cfg.nny):
        if ky == cfg.nny // 2:
            continue
        for kx in range(cfg.kx):
            a, b = ia[kx], ib[ky]
            k2 = a * a + b * b
            H1, H2, H3, V = h1[:, ky, kx], h2[:, ky, kx], h3[:, ky, kx], v[:, ky, kx]
            if k2 == 0.0:
                g = -H2
                c = np.zeros(n + 1, complex)
                for m in range(1, n + 1):
                    am1 = g[m - 1] * (2.0 if m == 1 else 1.0)
                    ap1 = g[m + 1] if m + 1 <= n else 0.0
                    c[m] = (am1 - ap1) / (2.0 * m)
                even = np.arange(2, n + 1, 2)
                c[0] = -np.sum(c[even] / (1.0 - even ** 2.0))
                P[:, ky, kx] = c
                continue
            g = -(1j * a * H1 + D @ H2 + 1j * b * H3)
            A = np.zeros((n + 1, n + 1))
            A[1:n] = (T2 - k2 * T0)[1:n]
            A[0], A[n] = top, bot
            rhs = np.zeros(n + 1, complex)
            rhs[1:n] = (T0 @ g)[1:n]
            w = -H2 + (D @ (D @ V) - k2 * V) / cfg.re
            rhs[0], rhs[n] = np.sum(w), np.sum(((-1.0) ** j) * w)
            P[:, ky, kx] = np.linalg.solve(A, rhs)
    out = np.empty(st["vnp1"].shape)
    out[:, :, 0::2], out[:, :, 1::2] = P.real, P.imag
    return out


@pytest.mark.parametrize("name", list(CASES))
def test_pressure_matches_dense_solve(chflow_lib, name):
    cfg = CASES[name]
    st = fields.turbulent_start_state(cfg, seed=6)
    ref = pressure_ref(cfg, st)
    outs = []
    for prec in ("fp64", "mixed"):
        with Channel(cfg, precision=prec) as g:
            g.upload_state(st)
            outs.append(g.pressure())
    nyq = cfg.nny // 2
    for got in outs:
        got[:, nyq, :] = 0.0
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err < 1e-10, err
    assert np.array_equal(outs[0], outs[1])  # FP64 for either precision


def test_laminar_pressure(chflow_lib):
    """U = g (1 - z^2): P = U^2 / 2 up to a constant, i.e. P_00 = -g^2 (5 T0 + 4 T2 - T4) / 16
    + 7 g^2 / 30 with zero mean; every other mode zero."""
    cfg = config.CONFIGS["c1_poiseuille_32"]
    for gamma in (1.0, 1.7):
        st = fields.laminar_state(cfg, gamma=gamma)
        with Channel(cfg) as g:
            g.upload_state(st)
            p = g.pressure()
        expect = np.zeros(cfg.nnz + 1)
        expect[0], expect[2], expect[4] = -19.0 / 240.0, -0.25, 1.0 / 16.0
        assert np.allclose(p[:, 0, 0], gamma ** 2 * expect, rtol=0, atol=1e-13)
        q = p.copy()
        q[:, 0, 0] = 0.0
        assert np.abs(q).max() < 1e-13
