"""The physical-space side of statistics on the GPU, through the C ABI:
transform (poiseuilleflow.f90:919-1005) in both directions against the
oracle's restatement of it, the CFL numbers (:2866-2934) against NumPy on
the oracle's physical fields, and the 3Ddata velocity dump (:2745-2764)
against the same fields and the host reader of the files.

Bars: 1e-13 relative for the transforms (FP64 DFTs of lengths up to 768,
agreement to rounding); 1e-12 for the CFL numbers and the dump."""
import numpy as np
import pytest

from channel_flow_gb300 import Channel, ChannelError, config, fields, restart

pytestmark = pytest.mark.gpu

CASES = {
    "small16": config.small(nnx=16, nny=8, nnz=16, aphi=1.0, beta=0.5, dt=5e-4, re=180.0, re_p=1.0),
    "mixed_radix": config.small(nnx=24, nny=12, nnz=20, aphi=1.5, beta=0.75, dt=5e-4, re=300.0, re_p=1.0),
    "c2_os": config.CONFIGS["c2_orr_sommerfeld"],
    "grid128": config.small(nnx=128, nny=128, nnz=32, aphi=2.0, beta=2.0 / 3.0, dt=2e-4, re=180.0, re_p=1.0),
    "long_xz": config.small(nnx=384, nny=8, nnz=192, aphi=1.0, beta=0.5, dt=2e-4, re=550.0, re_p=1.0),
    "long_y": config.small(nnx=8, nny=384, nnz=16, aphi=1.0, beta=0.5, dt=2e-4, re=550.0, re_p=1.0),
}


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("name", list(CASES))
def test_transform_matches_oracle(chflow_lib, oracle_mod, name):
    cfg = CASES[name]
    o = oracle_mod.Oracle.from_config(cfg)
    rng = np.random.default_rng(1)
    spec = rng.standard_normal((cfg.nnz + 1, cfg.nny, cfg.nnx))
    phys = rng.standard_normal((cfg.nnz + 1, cfg.nny, cfg.nnx))
    with Channel(cfg, precision="mixed" if name == "grid128" else "fp64") as g:
        fwd = g.transform(1, spec)
        back = g.transform(-1, phys)
    assert rel(fwd, o.transform(1, spec)) < 1e-13
    assert rel(back, o.transform(-1, phys)) < 1e-13


@pytest.mark.parametrize("name", ["small16", "mixed_radix", "long_y"])
def test_transform_round_trip(chflow_lib, name):
    """Spectral -> physical -> spectral returns the coefficients, except the
    Nyquist modes transform drops and the imaginary part of the streamwise
    mean, which a real field cannot carry."""
    cfg = CASES[name]
    st = fields.turbulent_start_state(cfg, seed=2)
    spec = st["unp1"].copy()
    spec[:, cfg.nny // 2, :] = 0.0
    spec[:, :, 1] = 0.0
    with Channel(cfg) as g:
        back = g.transform(-1, g.transform(1, spec))
    assert rel(back, spec) < 1e-13


def stepped(cfg, precision="fp64", nsteps=5, seed=4):
    st = fields.turbulent_start_state(cfg, seed=seed)
    g = Channel(cfg, precision=precision)
    g.upload_state(st)
    g.getnonlinear(); g.solve(); g.step(nsteps)
    return g


def reference_cfl(cfg, u, v, w):
    """CFL_X, CFL_Y, CFL_Z as statistics forms them (poiseuilleflow.f90:2866-2934)."""
    pi2 = 2.0 * np.pi
    dx = cfg.aphi * pi2 / cfg.nnx
    ddz = cfg.beta * pi2 / cfg.nny
    ddy = np.pi / cfg.nnz
    nz = cfg.nnz
    dy = np.zeros(nz + 1)
    for k in range(1, nz // 2 + 1):
        dy[k] = -(np.cos(k * ddy) - np.cos((k - 1) * ddy))
        dy[nz - k] = dy[k]
    cfly = [np.abs(v[k]).max() * cfg.dt / dy[k] for k in range(1, nz)]
    return {"cfl_x": np.abs(u).max() * cfg.dt / dx, "cfl_y": max(cfly), "cfl_z": np.abs(w).max() * cfg.dt / ddz}


@pytest.mark.parametrize("name,precision", [("mixed_radix", "fp64"), ("grid128", "mixed"), ("c2_os", "fp64")])
def test_cfl_matches_reference_formula(chflow_lib, oracle_mod, name, precision):
    cfg = CASES[name]
    o = oracle_mod.Oracle.from_config(cfg)
    with stepped(cfg, precision) as g:
        st = g.download_state()
        got = g.cfl()
    u, v, w = (o.transform(1, st[k]) for k in ("unp1", "vnp1", "wnp1"))
    want = reference_cfl(cfg, u, v, w)
    for k in want:
        assert abs(got[k] - want[k]) <= 1e-12 * want[k], (k, got[k], want[k])


@pytest.mark.parametrize("nproc", [1, 2])
def test_velocity_dump(chflow_lib, oracle_mod, tmp_path, nproc):
    cfg = CASES["mixed_radix"]
    o = oracle_mod.Oracle.from_config(cfg)
    u0 = 0.1 * np.cos(np.pi * np.arange(cfg.nnz + 1) / cfg.nnz) ** 2
    with stepped(cfg) as g:
        st = g.download_state()
        vel = g.physical_velocity(u0)
        g.write_velocity(str(tmp_path), nproc=nproc, istep=1000, u0=u0)
        plain = g.physical_velocity()
        stats = g.statistics()
    u, v, w = (o.transform(1, st[k]) for k in ("unp1", "vnp1", "wnp1"))
    want = np.stack([u + u0[:, None, None], w, v])
    assert rel(vel, want) < 1e-12
    # the files hold exactly the returned array, slab by slab
    assert np.array_equal(restart.read_velocity_dump(cfg, str(tmp_path), istep=1000, nproc=nproc), vel)
    # the energy statistics prints from the dump (u0 = 0) equals the
    # spectral (Parseval) energy of chf_statistics
    e = 0.5 * float((plain ** 2).sum())
    assert abs(e - stats["energy"]) <= 1e-12 * e


def test_dump_rejects_bad_nproc(chflow_lib, tmp_path):
    cfg = CASES["mixed_radix"]  # nny / 2 = 6: 4 ranks cannot split it
    with stepped(cfg, nsteps=1) as g:
        with pytest.raises(ChannelError) as ei:
            g.write_velocity(str(tmp_path), nproc=4)
        assert ei.value.code == -1
