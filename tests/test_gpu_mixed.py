"""Mixed-precision path (FP32 transforms and products, bf16x3 tcgen05 GEMMs
for the wall-normal transforms, FP64 implicit solves) against the FP64 path
and the oracle.  Bar: velocity rel-L2 <= 1e-5 against FP64 (the accuracy the
mixed form must hold); the nonlinear term itself to 1e-5 after one call."""
import numpy as np
import pytest

from channel_flow_gb300 import Channel, config, fields
from parity import compare, rel_l2, split

pytestmark = pytest.mark.gpu

CASES = {
    "small16": config.small(nnx=16, nny=8, nnz=16, aphi=1.0, beta=0.5, dt=5e-4, re=180.0, re_p=1.0),
    "c1_32": config.CONFIGS["c1_poiseuille_32"],
    "c2_os": config.CONFIGS["c2_orr_sommerfeld"],
    "mixed_radix": config.small(nnx=24, nny=12, nnz=20, aphi=1.5, beta=0.75, dt=5e-4, re=300.0, re_p=1.0),
    "warp192": config.small(nnx=128, nny=128, nnz=16, aphi=2.0, beta=2.0 / 3.0, dt=2e-4, re=180.0, re_p=1.0),
    "long_xz": config.small(nnx=384, nny=8, nnz=192, aphi=1.0, beta=0.5, dt=2e-4, re=550.0, re_p=1.0),
    "long_y": config.small(nnx=8, nny=384, nnz=16, aphi=1.0, beta=0.5, dt=2e-4, re=550.0, re_p=1.0),
    # the largest wall-normal degree (251 points): K = 256 digit rows in Z1 (four planes)
    "tall_z": config.small(nnx=8, nny=8, nnz=250, aphi=1.0, beta=0.5, dt=1e-4, re=550.0, re_p=1.0),
}
VEL = ("unp1", "vnp1", "wnp1")


def vel_err(a, b):
    out = {}
    for k in VEL:
        pa, pb = split(a[k], k)[k], split(b[k], k)[k]
        out[k] = rel_l2(pa, pb)
    return out


def run(cfg, st, precision, nsteps, zpad=0):
    with Channel(cfg, precision=precision, zpad=zpad) as g:
        g.upload_state(st)
        g.getnonlinear()
        g.solve()
        g.step(nsteps)
        g.synchronize()
        return g.download_state()


@pytest.mark.parametrize("name", list(CASES))
def test_mixed_nonlinear_term(chflow_lib, name):
    cfg = CASES[name]
    st = fields.turbulent_start_state(cfg, seed=2)
    outs = {}
    for prec in ("fp64", "mixed"):
        with Channel(cfg, precision=prec) as g:
            g.upload_state(st)
            g.getnonlinear()
            g.synchronize()
            outs[prec] = g.download_state()
    for k in ("rhsvn", "rhsomegayn"):
        e = rel_l2(split(outs["mixed"][k], k)[k], split(outs["fp64"][k], k)[k])
        assert e < 1e-5, (k, e)
    for k in ("clamb1n", "clamb3n"):
        e = np.linalg.norm(outs["mixed"][k] - outs["fp64"][k]) / max(np.linalg.norm(outs["fp64"][k]), 1e-30)
        assert e < 1e-4, (k, e)


@pytest.mark.parametrize("precision", ["mixed", "mixed_fp64solve"])
@pytest.mark.parametrize("name,nsteps", [("small16", 50), ("c1_32", 50), ("c2_os", 50), ("mixed_radix", 30),
                                          ("warp192", 30), ("long_xz", 10), ("long_y", 20), ("tall_z", 10)])
def test_mixed_steps_vs_fp64(chflow_lib, name, nsteps, precision):
    cfg = CASES[name]
    st = fields.turbulent_start_state(cfg, seed=4)
    a = run(cfg, st, "fp64", nsteps)
    b = run(cfg, st, precision, nsteps)
    errs = vel_err(b, a)
    assert max(errs.values()) < 1e-5, errs


def test_fp64solve_form_runs_the_fp64_solve(chflow_lib):
    """CHF_MIXED_F64SOLVE shares the nonlinear term of CHF_MIXED and the
    solve of CHF_FP64: one solve from the same post-nonlinear state is
    bit-identical to the FP64 path's."""
    cfg = CASES["mixed_radix"]
    st = fields.turbulent_start_state(cfg, seed=8)
    with Channel(cfg, precision="mixed_fp64solve") as g:
        g.upload_state(st)
        g.getnonlinear()
        mid = g.download_state()
        g.solve()
        got = g.download_state()
    with Channel(cfg, precision="fp64") as f:
        f.upload_state(mid)
        f.solve()
        want = f.download_state()
    for k in ("vnp1", "omegaynp1", "unp1", "wnp1", "omegaxnp1", "omegaznp1", "au0", "w0"):
        assert np.array_equal(got[k], want[k]), k


def test_mixed_steps_vs_oracle(chflow_lib, oracle_mod):
    cfg = CASES["c1_32"]
    st = fields.lowmode_state(cfg, seed=5, amp=1e-2)
    o = oracle_mod.Oracle.from_config(cfg)
    o.setup()
    o.set_state(st)
    o.getnonlinear(); o.solve(); o.step(40)
    b = run(cfg, st, "mixed", 40)
    errs = vel_err(b, o.get_state())
    assert max(errs.values()) < 1e-5, errs


def test_mixed_zpad_auto_matches_default(chflow_lib):
    cfg = CASES["small16"]
    st = fields.turbulent_start_state(cfg, seed=6)
    a = run(cfg, st, "mixed", 10, zpad=0)
    b = run(cfg, st, "mixed", 10, zpad=25)
    errs = vel_err(b, a)
    assert max(errs.values()) < 1e-6, errs


def test_mixed_full_size(chflow_lib):
    cfg = config.CONFIGS["c3_retau180_128"]
    st = fields.turbulent_start_state(cfg, seed=1)
    a = run(cfg, st, "fp64", 20, zpad=200)
    b = run(cfg, st, "mixed", 20, zpad=200)
    errs = vel_err(b, a)
    assert max(errs.values()) < 1e-5, errs


def test_mixed_retau550_full_size(chflow_lib):
    """The Re_tau 550 box, 384 x 193 x 384 on the exact 300-interval product
    grid (2 * 300 > 3 * 192): both paths run it, and agree."""
    cfg = config.CONFIGS["c4_retau550_384"]
    st = fields.turbulent_start_state(cfg, seed=1)
    a = run(cfg, st, "fp64", 5, zpad=300)
    assert all(np.isfinite(a[k]).all() for k in VEL)
    b = run(cfg, st, "mixed", 5, zpad=300)
    errs = vel_err(b, a)
    assert max(errs.values()) < 1e-5, errs


@pytest.fixture(scope="module")
def fp64_after_1000():
    cfg = config.CONFIGS["c3_retau180_128"]
    st = fields.turbulent_start_state(cfg, seed=0)
    return cfg, st, run(cfg, st, "fp64", 1000, zpad=200)


@pytest.mark.parametrize("precision", ["mixed", "mixed_fp64solve"])
def test_mixed_accuracy_after_1000_steps(chflow_lib, fp64_after_1000, precision):
    """The mixed forms' accuracy target at Re_tau 180, 128 x 129 x 128: the
    velocity (u, v, w) rel-L2 against the FP64 path after 1000 steps from the
    same start is at most 1e-5."""
    cfg, st, a = fp64_after_1000
    b = run(cfg, st, precision, 1000, zpad=200)
    num = den = 0.0
    for k in VEL:
        pa, pb = split(a[k], k)[k], split(b[k], k)[k]
        num += float(np.sum((pb - pa) ** 2))
        den += float(np.sum(pa ** 2))
    vel = (num / den) ** 0.5
    assert vel <= 1e-5, (vel, vel_err(b, a))


@pytest.mark.parametrize("precision", ["mixed", "mixed_fp64solve"])
@pytest.mark.parametrize("name", ["small16", "c1_32", "mixed_radix"])
def test_mixed_from_reference_initial_field(chflow_lib, name, precision):
    """The analytic-plus-point-noise start of the reference's input
    (poiseuilleflow.f90:2086-2339): white noise in every mode, and a wall
    slope of v that the first solve has to remove (the reference's wall rows
    hold the boundary values).  Both mixed forms follow the FP64 path."""
    cfg = CASES[name]
    st = fields.reference_like_state(cfg, seed=3, epsilon=0.3, noise=0.02, gamma=5.0)
    a = run(cfg, st, "fp64", 5)
    b = run(cfg, st, precision, 5)
    errs = vel_err(b, a)
    assert max(errs.values()) < 1e-5, errs


@pytest.mark.parametrize("form", ["fp64", "mixed/fp64 recovery", "mixed/double-float recovery"])
@pytest.mark.parametrize("name", ["small16", "mixed_radix", "long_xz", "warp192"])
def test_mixed_recovery_matches_fp64(chflow_lib, name, form):
    """The recovery of u, w, omega_x, omega_z from v and omega_y after three
    steps (k_inc_recover64 in FP64, k_inc_recover in double-float, about
    2^-44; the FP64 path's own in k_solve) against getvelocityandvorticity in
    FP64 NumPy applied to the same v and omega_y: to 1e-11 relative (FP32
    arithmetic would leave about 1e-6)."""
    cfg = CASES[name]
    st = fields.turbulent_start_state(cfg, seed=21)
    precision = form.split("/")[0]
    with Channel(cfg, precision=precision) as g:
        if precision == "mixed":
            g.set_launch_shape("recover_form", 1 if "double" in form else 0)
        g.upload_state(st)
        g.getnonlinear()
        g.solve()
        g.step(3)
        out = g.download_state()
    ref = {k: v.copy() for k, v in out.items()}
    fields.recover_velocity(cfg, ref)
    nyq = cfg.nny // 2
    for k in ("unp1", "wnp1", "omegaxnp1", "omegaznp1"):
        a, b = out[k].copy(), ref[k].copy()
        a[:, nyq, :] = 0.0
        b[:, nyq, :] = 0.0
        e = rel_l2(a, b)
        assert e < 1e-11, (k, e)
