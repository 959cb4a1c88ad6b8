"""The CPU oracle against independent checks (no GPU): NumPy's FFT, exact
Chebyshev calculus, the reference's own A * inv(A) self-check, known
answers, and the committed golden fixtures (extended-precision Lamb vectors,
oracle steps)."""
import os

import numpy as np
import pytest

from channel_flow_gb300 import config, fields
from exact_lamb import lamb
from parity import FIELD_NAMES, MEAN_NAMES, compare

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SMALL = config.small(nnx=16, nny=8, nnz=16, aphi=1.0, beta=0.5, dt=5e-4, re=180.0, re_p=1.0)


@pytest.mark.parametrize("n", [4, 6, 12, 48, 192, 256, 384, 400, 512, 10])
def test_fft_matches_numpy(oracle_mod, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    assert np.abs(oracle_mod.fft(x, -1) - np.fft.fft(x)).max() < 1e-13 * n
    assert np.abs(oracle_mod.fft(x, +1) - np.fft.ifft(x) * n).max() < 1e-13 * n


@pytest.mark.parametrize("n", [4, 16, 33, 128])
def test_dz_is_chebyshev_derivative(oracle_mod, n):
    c = np.random.default_rng(n).standard_normal(n + 1)
    d = oracle_mod.dz(c)
    ref = np.polynomial.chebyshev.chebder(c)
    assert np.allclose(d[:n], ref, rtol=1e-13, atol=1e-12 * np.abs(ref).max())
    assert d[n] == 0.0


def test_inverse_self_check(oracle_mod):
    """A * inv(A) = I, the check the reference prints at poiseuilleflow.f90:206-212."""
    cfg = config.CONFIGS["c3_retau180_128"]
    o = oracle_mod.Oracle.from_config(cfg)
    for k2 in (0.25, 1.0, 97.25, 4000.0):
        av, ae, xv, xe = o.matrices(k2)
        assert np.abs(av @ xv - np.eye(cfg.nnz + 1)).max() < 1e-9
        assert np.abs(ae @ xe - np.eye(cfg.nnz + 1)).max() < 1e-13


def test_scheb_matches_chebyshev_polynomials(oracle_mod):
    o = oracle_mod.Oracle.from_config(SMALL)
    t0, t1, t2, t4 = o.scheb()
    n = SMALL.nnz
    z = fields.zpoints(n)
    for L in range(n + 1):
        c = np.zeros(n + 1)
        c[L] = 1.0
        assert np.allclose(t0[:, L], np.polynomial.chebyshev.chebval(z, c), atol=1e-12)
        d1 = np.polynomial.chebyshev.chebder(c, 1)
        d2 = np.polynomial.chebyshev.chebder(c, 2)
        d4 = np.polynomial.chebyshev.chebder(c, 4)
        scale = max(1.0, L ** 4)
        assert np.allclose(t1[:, L], np.polynomial.chebyshev.chebval(z, d1), atol=1e-9 * scale)
        assert np.allclose(t2[:, L], np.polynomial.chebyshev.chebval(z, d2), atol=1e-9 * scale)
        if L >= 4:
            assert np.allclose(t4[1:n, L], np.polynomial.chebyshev.chebval(z[1:n], d4), rtol=1e-8,
                               atol=1e-8 * L ** 8)


def test_laminar_fixed_point(oracle_mod):
    cfg = config.CONFIGS["c1_poiseuille_32"]
    st = fields.laminar_state(cfg)
    o = oracle_mod.Oracle.from_config(cfg)
    o.setup()
    o.set_state(st)
    o.step(20)
    for k in ("au0", "unp1", "omegaznp1"):
        assert np.abs(o.get_state()[k] - st[k]).max() < 1e-12 * np.abs(st[k]).max()


def test_spectral_round_trip(oracle_mod):
    o = oracle_mod.Oracle.from_config(SMALL)
    rng = np.random.default_rng(0)
    sp = rng.standard_normal((SMALL.nnz + 1, SMALL.nny, SMALL.nnx))
    sp[:, SMALL.nny // 2, :] = 0.0
    sp[:, 0, 1] = 0.0  # the imaginary part of the streamwise mean is dropped by c2r
    # make kx = 0 Hermitian in ky so the physical field is real
    c = fields.as_complex(sp)
    for j in range(1, SMALL.nny // 2):
        c[:, SMALL.nny - j, 0] = np.conj(c[:, j, 0])
    back = o.transform(-1, o.transform(1, sp))
    assert np.abs(back - sp).max() < 1e-14 * np.abs(sp).max() * 10


def test_host_phys_to_spec_matches_oracle_transform(oracle_mod):
    o = oracle_mod.Oracle.from_config(SMALL)
    f = np.random.default_rng(1).standard_normal((SMALL.nnz + 1, SMALL.nny, SMALL.nnx))
    assert np.abs(fields.phys_to_spec(SMALL, f) - o.transform(-1, f)).max() < 1e-14


@pytest.mark.parametrize("name", ["tiny8", "tiny12"])
def test_golden_lamb(oracle_mod, name):
    g = np.load(os.path.join(GOLDEN, f"lamb_{name}.npz"))
    from golden.make_golden import CASES
    cfg = CASES[name]
    st = {k[3:]: g[k] for k in g.files if k.startswith("in_")}
    o = oracle_mod.Oracle.from_config(cfg)
    h1 = o.getlamb(st["omegaynp1"], st["wnp1"], True) - o.getlamb(st["omegaznp1"], st["vnp1"], False)
    h2 = o.getlamb(st["omegaznp1"], st["unp1"], False) - o.getlamb(st["omegaxnp1"], st["wnp1"], False)
    h3 = o.getlamb(st["omegaxnp1"], st["vnp1"], False) - o.getlamb(st["omegaynp1"], st["unp1"], False)
    for got, key in ((h1, "h1"), (h2, "h2"), (h3, "h3")):
        ex = g[key]
        assert np.linalg.norm(got - ex) / np.linalg.norm(ex) < 1e-12, key


def test_exact_lamb_reproduces_golden():
    g = np.load(os.path.join(GOLDEN, "lamb_tiny8.npz"))
    from golden.make_golden import CASES
    cfg = CASES["tiny8"]
    st = {k[3:]: g[k] for k in g.files if k.startswith("in_")}
    h1, h2, h3 = lamb(cfg, st)
    assert np.array_equal(h1, g["h1"]) and np.array_equal(h3, g["h3"])


@pytest.mark.parametrize("name", ["tiny8", "tiny12"])
def test_golden_steps(oracle_mod, name):
    g = np.load(os.path.join(GOLDEN, f"steps_{name}.npz"))
    from golden.make_golden import CASES
    cfg = CASES[name]
    st = {k[3:]: g[k] for k in g.files if k.startswith("in_")}
    o = oracle_mod.Oracle.from_config(cfg)
    o.setup()
    o.set_state(st)
    o.getnonlinear()
    o.solve()
    o.step(1)
    ref = {k[3:]: g[k] for k in g.files if k.startswith("s1_")}
    errs = compare(o.get_state(), ref, names=FIELD_NAMES + MEAN_NAMES)
    assert max(errs.values()) < 1e-12, errs


TALL = config.small(nnx=8, nny=8, nnz=250, aphi=1.0, beta=0.5, dt=1e-4, re=550.0, re_p=1.0)


@pytest.mark.parametrize("cfg,bar", [(SMALL, 1e-12), (config.CONFIGS["c1_poiseuille_32"], 1e-12)])
def test_extended_histories_match_oracle(oracle_mod, cfg, bar):
    """The extended-precision curl and Gauss-Lobatto values (the reference the
    GPU histories are held to at the largest degree) agree with the oracle's
    getnonlinear where both are accurate."""
    from exact_lamb import nonlinear_histories
    from parity import rel_l2, split
    st = fields.reference_like_state(cfg, seed=3, epsilon=0.3, noise=0.02, gamma=5.0)
    ev, eg = nonlinear_histories(cfg, st)
    o = oracle_mod.Oracle.from_config(cfg)
    o.setup()
    o.set_state(st)
    o.getnonlinear()
    got = o.get_state()
    for k, ex in (("rhsvn", ev), ("rhsomegayn", eg)):
        assert rel_l2(split(got[k], k)[k], split(ex, k)[k]) < bar, k


def test_largest_degree_oracle_accuracy(oracle_mod):
    """At nnz = 250 the reference algorithm's nonlinear histories are only
    ~1e-8 accurate (the derivative of the curl amplifies the products'
    rounding), and the v operator is ill-conditioned (~3e9): the facts the GPU
    parity bars at that degree rest on."""
    from exact_lamb import nonlinear_histories
    from parity import rel_l2, split
    st = fields.reference_like_state(TALL, seed=3, epsilon=0.3, noise=0.02, gamma=5.0)
    ev, eg = nonlinear_histories(TALL, st)
    o = oracle_mod.Oracle.from_config(TALL)
    o.setup()
    o.set_state(st)
    o.getnonlinear()
    got = o.get_state()
    ev_err = rel_l2(split(got["rhsvn"], "rhsvn")["rhsvn"], split(ev, "rhsvn")["rhsvn"])
    eg_err = rel_l2(split(got["rhsomegayn"], "rhsomegayn")["rhsomegayn"], split(eg, "rhsomegayn")["rhsomegayn"])
    assert 1e-9 < ev_err < 1e-6 and 1e-9 < eg_err < 1e-6, (ev_err, eg_err)
    av, ae, xv, xe = o.matrices(17.0)
    assert 1e9 < np.linalg.cond(av) < 1e10
    assert np.linalg.cond(ae) < 100.0
    assert np.linalg.norm(av @ xv - np.eye(av.shape[0])) < 1e-9
