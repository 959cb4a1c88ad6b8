"""FP64 CUDA path vs the CPU oracle, through the C ABI.

Tolerances: per-array relative L2 error.  One getnonlinear, one solve
or N full steps: 1e-10 (the bar the FP64 path must meet against the
reference algorithm).  The (0,0)-mode Lamb histories clamb* are plane
averages with heavy cancellation; the oracle itself is 1e-11..1e-9 away from
their extended-precision value, so they are held to 1e-7 here and, in
test_mean_lamb_accuracy, the GPU must be at least as accurate as the oracle.  The GPU evaluates the same mathematics with a
different operation order (6+3 instead of 12+6 transforms, even/odd block
inverses, recurrence-based explicit terms), so agreement is to rounding, not
bitwise.
"""
import numpy as np
import pytest

from channel_flow_gb300 import Channel, ChannelError, config, fields
from channel_flow_gb300.fields import FIELD_NAMES, MEAN_NAMES
from exact_lamb import lamb, nonlinear_histories
from exact_mean import mean_h1
from parity import PROG, bad_parts, check, compare, oracle_sensitivity, rel_l2, split, worst

pytestmark = pytest.mark.gpu

CASES = {
    "small16": config.small(nnx=16, nny=8, nnz=16, aphi=1.0, beta=0.5, dt=5e-4, re=180.0, re_p=1.0),
    "c1_32": config.CONFIGS["c1_poiseuille_32"],
    "c2_os": config.CONFIGS["c2_orr_sommerfeld"],
    "mixed_radix": config.small(nnx=24, nny=12, nnz=20, aphi=1.5, beta=0.75, dt=5e-4, re=300.0, re_p=1.0),
    # 3/2-padded lengths of 192: the register-FFT kernels of the 128-point directions
    "warp192": config.small(nnx=128, nny=128, nnz=16, aphi=2.0, beta=2.0 / 3.0, dt=2e-4, re=180.0, re_p=1.0),
    # the long lines of the Re_tau 550 box (384 x 193 x 384): 576-point x rows
    # and 768-point z lines (fewer lines per CTA), and 576-point y lines
    "long_xz": config.small(nnx=384, nny=8, nnz=192, aphi=1.0, beta=0.5, dt=2e-4, re=550.0, re_p=1.0),
    "long_y": config.small(nnx=8, nny=384, nnz=16, aphi=1.0, beta=0.5, dt=2e-4, re=550.0, re_p=1.0),
    # the largest wall-normal degree chf_create accepts (251 points, 500-point z lines)
    "tall_z": config.small(nnx=8, nny=8, nnz=250, aphi=1.0, beta=0.5, dt=1e-4, re=550.0, re_p=1.0),
}


# Cases where the reference algorithm (the oracle) is itself far from exact
# in the nonlinear histories: at nnz = 250 its rhsvn / rhsomegayn are 2.4e-8 /
# 7.5e-8 from an extended-precision evaluation (the derivative of the curl
# multiplies the products' rounding by up to 2 nnz) and its plane-averaged H1
# 1.8e-6.  There the GPU's histories are held to that evaluation instead, at
# least as accurate as the oracle's (test_mean_lamb_accuracy for the (0,0)
# mode).
EXACT_HIST = ("tall_z",)

# Per-case bar of the prognostic arrays after one solve.  tall_z: the v
# operator's condition number is 3.4e9 at nnz = 250 (4.3e8 at 192); the
# oracle's explicit FP64 inverse leaves |A X - I| = 1.8e-10, so two
# independent eliminations (full LU here, even/odd Gauss-Jordan on the GPU)
# agree in v to about 1e-9 (omega_y, condition 28, to 1e-15).
SOLVE_TOL = {"tall_z": 1e-8}


def exact_zpad(n):
    """Smallest 2,3,5-smooth M with 2M > 3n: the smallest exact product grid."""
    m = 3 * n // 2 + 1
    while True:
        r = m
        for p in (2, 3, 5):
            while r % p == 0:
                r //= p
        if r == 1:
            return m
        m += 1


def make_state(cfg, seed=3):
    return fields.reference_like_state(cfg, seed=seed, epsilon=0.3, noise=0.02, gamma=5.0)


def make_smooth_state(cfg, seed=3):
    return fields.turbulent_start_state(cfg, seed=seed)


def pair(cfg, oracle_mod, st, zpad=0):
    o = oracle_mod.Oracle.from_config(cfg)
    o.setup()
    o.set_state(st)
    g = Channel(cfg, zpad=zpad)
    g.upload_state(st)
    return o, g


@pytest.mark.parametrize("name", list(CASES))
def test_upload_download_roundtrip(chflow_lib, name):
    cfg = CASES[name]
    rng = np.random.default_rng(0)
    st = {k: rng.standard_normal((cfg.nnz + 1, cfg.nny, cfg.nnx)) for k in FIELD_NAMES}
    st.update({k: rng.standard_normal((cfg.nnz + 1, 2)) for k in MEAN_NAMES})
    with Channel(cfg) as g:
        g.upload_state(st)
        back = g.download_state()
    for k in st:
        assert np.array_equal(back[k], st[k]), k


@pytest.mark.parametrize("name", list(CASES))
def test_getnonlinear_matches_oracle(chflow_lib, oracle_mod, name):
    cfg = CASES[name]
    st = make_state(cfg)
    o, g = pair(cfg, oracle_mod, st)
    o.getnonlinear()
    g.getnonlinear()
    gs, os_ = g.download_state(), o.get_state()
    # omega_x / omega_z now hold H1 / H3, whose accuracy is pinned against
    # extended precision in test_lamb_accuracy; every other array here
    for k in ("omegaxnp1", "omegaznp1"):
        gs.pop(k)
        os_.pop(k)
    hist = ("rhsvn", "rhsomegayn", "clamb1n", "clamb3n") if name in EXACT_HIST else ()
    names = tuple(k for k in os_ if k not in hist)
    errs = compare(gs, os_, names=names)
    bad = bad_parts(errs, 1e-10, 1e-7)
    if bad:
        # e.g. 384-point x rows: h_g mixes alpha up to 191 with small H, a
        # condition of ~5e5 (one-ulp input noise moves the oracle by 1e-10)
        floor = oracle_sensitivity(oracle_mod, cfg, st, lambda o: o.getnonlinear(), names=names)
        bad = bad_parts(errs, 1e-10, 1e-7, floor)
    assert not bad, (bad, errs)
    if hist:
        ev, eg = nonlinear_histories(cfg, st)
        for k, ex in (("rhsvn", ev), ("rhsomegayn", eg)):
            e_g = rel_l2(split(gs[k], k)[k], split(ex, k)[k])
            e_o = rel_l2(split(os_[k], k)[k], split(ex, k)[k])
            assert e_g <= max(2.0 * e_o, 1e-12), (k, e_g, e_o)


@pytest.mark.parametrize("name", ["small16", "c2_os", "mixed_radix"])
def test_lamb_accuracy(chflow_lib, oracle_mod, name):
    """H1, H3 (left in omega_x, omega_z by getnonlinear, REF:1489-1496)
    against an extended-precision evaluation of the dealiased products: the
    GPU must be at least as accurate as the reference algorithm (the oracle
    is 2e-10 off for the Orr-Sommerfeld box, whose H1 is a near-cancelling
    sum)."""
    cfg = CASES[name]
    st = make_state(cfg)
    h1, h2, h3 = lamb(cfg, st)
    o, g = pair(cfg, oracle_mod, st)
    o.getnonlinear()
    g.getnonlinear()
    out = g.download_state()
    for key, ex in (("omegaxnp1", h1), ("omegaznp1", h3)):
        e_o = np.linalg.norm(o.field(key) - ex) / np.linalg.norm(ex)
        e_g = np.linalg.norm(out[key] - ex) / np.linalg.norm(ex)
        assert e_g <= max(2.0 * e_o, 1e-13), (key, e_g, e_o)


@pytest.mark.parametrize("name", list(CASES))
def test_solve_matches_oracle(chflow_lib, oracle_mod, name):
    cfg = CASES[name]
    st = make_state(cfg, seed=5)
    o, g = pair(cfg, oracle_mod, st)
    o.getnonlinear()
    mid = o.get_state()
    g.upload_state(mid)
    o.solve()
    g.solve()
    check(g.download_state(), o.get_state(), SOLVE_TOL.get(name, 1e-10), 1e-7)


# Per-case bar for the prognostic arrays after several steps.  long_xz: the
# reference algorithm's plane average H(0,0) on this 384-point box is only
# ~2.5e-8 accurate against extended precision (the GPU's is pinned to be at
# least as accurate in test_mean_lamb_accuracy[long_xz]); the mean spanwise
# flow w0 and, through it, the nonlinear histories inherit that difference.
STEP_TOL = {"long_xz": 1e-8}


@pytest.mark.parametrize("name,nsteps", [("small16", 40), ("c1_32", 20), ("c2_os", 20), ("mixed_radix", 20),
                                          ("warp192", 10), ("long_xz", 3), ("long_y", 5)])
def test_steps_match_oracle(chflow_lib, oracle_mod, name, nsteps):
    cfg = CASES[name]
    st = make_state(cfg, seed=7)
    o, g = pair(cfg, oracle_mod, st)
    # the reference's start-up: getnonlinear in initial(), then a solve-only step
    o.getnonlinear(); o.solve()
    g.getnonlinear(); g.solve()
    o.step(nsteps)
    g.step(nsteps)

    def run(o):
        o.getnonlinear()
        o.solve()
        o.step(nsteps)

    gs = g.download_state()

    def floor():
        # rounding-level spread of the result: the oracle's response to
        # one-ulp input noise, and the GPU path on another exact product
        # grid (same mathematics, different rounding)
        f = oracle_sensitivity(oracle_mod, cfg, st, run)
        with Channel(cfg, zpad=exact_zpad(cfg.nnz)) as g2:
            g2.upload_state(st)
            g2.getnonlinear(); g2.solve()
            g2.step(nsteps)
            alt = compare(g2.download_state(), gs)
        return {k: max(f.get(k, 0.0), alt.get(k, 0.0)) for k in set(f) | set(alt)}

    check(gs, o.get_state(), STEP_TOL.get(name, 1e-10), 1e-7, sensitivity=floor)


def test_lowmode_c1_steps(chflow_lib, oracle_mod):
    cfg = CASES["c1_32"]
    st = fields.lowmode_state(cfg, seed=11, amp=1e-3)
    o, g = pair(cfg, oracle_mod, st)
    o.getnonlinear(); o.solve(); o.step(30)
    g.getnonlinear(); g.solve(); g.step(30)
    check(g.download_state(), o.get_state(), 1e-10, 1e-7)


def test_zpad_equivalence(chflow_lib):
    """Any product grid with 2*zpad > 3*nnz gives the same products."""
    cfg = CASES["small16"]
    st = make_state(cfg, seed=9)
    outs = []
    for zpad in (0, 25, 27, 40):
        with Channel(cfg, zpad=zpad) as g:
            g.upload_state(st)
            g.getnonlinear(); g.solve(); g.step(5)
            outs.append(g.download_state())
    for other in outs[1:]:
        k, e = worst(compare(other, outs[0]))
        assert e < 1e-12, (k, e)


def test_laminar_fixed_point(chflow_lib):
    cfg = CASES["c1_32"]
    st = fields.laminar_state(cfg)
    with Channel(cfg) as g:
        g.upload_state(st)
        g.step(50)
        out = g.download_state()
    for k in ("au0", "unp1", "omegaznp1", "clamb1n", "clamb1nm1"):
        err = np.abs(out[k] - st[k]).max() / max(np.abs(st[k]).max(), 1.0)
        assert err < 1e-11, (k, err)


def test_diagnostics_energy(chflow_lib):
    cfg = CASES["c1_32"]
    st = make_state(cfg)
    with Channel(cfg) as g:
        g.upload_state(st)
        d = g.diagnostics()
    nyq = cfg.nny // 2
    e = 0.5 * sum((np.delete(st[k], nyq, axis=1) ** 2).sum() for k in ("unp1", "vnp1", "wnp1"))
    assert d["finite"]
    assert abs(d["energy"] - e) <= 1e-12 * e
    mx = max(np.abs(np.delete(st[k], nyq, axis=1)).max() for k in FIELD_NAMES[:6])
    assert d["max_abs"] == mx


def test_nonfinite_state_is_reported(chflow_lib):
    cfg = CASES["small16"]
    st = make_state(cfg)
    st["vnp1"][3, 2, 1] = np.nan
    with Channel(cfg) as g:
        g.upload_state(st)
        d = g.diagnostics()
    assert not d["finite"]


def test_step_before_upload_is_an_error(chflow_lib):
    with Channel(CASES["small16"]) as g:
        with pytest.raises(ChannelError) as ei:
            g.step(1)
        assert ei.value.code == -4


def test_divergence_free_after_steps(chflow_lib):
    """i alpha u + Dv + i beta w = 0 for every solved mode (REF:2365-2377)."""
    cfg = CASES["c1_32"]
    st = make_state(cfg)
    with Channel(cfg) as g:
        g.upload_state(st)
        g.getnonlinear(); g.solve(); g.step(5)
        out = g.download_state()
    ia, ib = fields.wavenumbers(cfg)
    D = fields.cheb_derivative_matrix(cfg.nnz)
    u = fields.as_complex(out["unp1"]); v = fields.as_complex(out["vnp1"]); w = fields.as_complex(out["wnp1"])
    div = 1j * ia[None, None, :] * u + np.tensordot(D, v, axes=(1, 0)) + 1j * ib[None, :, None] * w
    div[:, cfg.nny // 2, :] = 0
    div[:, 0, 0] = 0
    scale = np.abs(np.tensordot(D, v, axes=(1, 0))).max()
    assert np.abs(div).max() < 1e-11 * scale


def test_full_size_two_steps(chflow_lib, oracle_mod):
    """128 x 129 x 128 (Re_tau 180 box): two full steps against the oracle."""
    cfg = config.CONFIGS["c3_retau180_128"]
    st = make_smooth_state(cfg, seed=1)
    o, g = pair(cfg, oracle_mod, st)
    o.getnonlinear(); o.solve(); o.step(1)
    g.getnonlinear(); g.solve(); g.step(1)
    check(g.download_state(), o.get_state(), 1e-10, 1e-6)


@pytest.mark.parametrize("name", ["c1_32", "c2_os", "small16", "long_xz", "tall_z"])
def test_mean_lamb_accuracy(chflow_lib, oracle_mod, name):
    """H1(0,0) (left in omegaxnp1 by getnonlinear, REF:1489-1496) against its
    extended-precision value: the GPU must be at least as accurate as the
    reference algorithm."""
    cfg = CASES[name]
    st = make_state(cfg)
    exact = mean_h1(cfg, st)
    o, g = pair(cfg, oracle_mod, st)
    o.getnonlinear()
    g.getnonlinear()
    got_o = o.field("omegaxnp1")[:, 0, 0] + 1j * o.field("omegaxnp1")[:, 0, 1]
    out = g.download_state()["omegaxnp1"]
    got_g = out[:, 0, 0] + 1j * out[:, 0, 1]
    err_o = np.linalg.norm(got_o - exact) / np.linalg.norm(exact)
    err_g = np.linalg.norm(got_g - exact) / np.linalg.norm(exact)
    assert err_g <= max(2.0 * err_o, 1e-13), (err_g, err_o)


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_fp64solve"])
def test_step_graph_matches_direct_launches(chflow_lib, precision):
    """chf_step replays a captured graph for pairs of steps; the state after
    7 steps (3 replays and one direct step) is bit-identical to 7 direct
    getnonlinear + solve calls, and to a second handle stepping 3 + 4."""
    cfg = CASES["mixed_radix"]
    st = make_state(cfg, seed=9)
    with Channel(cfg, precision=precision) as a, Channel(cfg, precision=precision) as b, \
            Channel(cfg, precision=precision) as c:
        for g in (a, b, c):
            g.upload_state(st)
        a.step(7)
        for _ in range(7):
            b.getnonlinear()
            b.solve()
        c.step(3)
        c.step(4)
        outs = [g.download_state() for g in (a, b, c)]
    for k in FIELD_NAMES + MEAN_NAMES:
        assert np.array_equal(outs[0][k], outs[1][k]), k
        assert np.array_equal(outs[0][k], outs[2][k]), k
