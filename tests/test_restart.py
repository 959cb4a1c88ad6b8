"""Restart files in the reference's layout (host side, no GPU): round trips
over nproc slabs, the byte layout of the Fortran records, and rejection of
layouts the reference cannot run."""
import os

import numpy as np
import pytest

from channel_flow_gb300 import config, fields, restart

CFG = config.small(nnx=16, nny=8, nnz=8, aphi=1.0, beta=0.5, dt=1e-3, re=100.0, re_p=1.0)


def state(seed=0):
    st = fields.reference_like_state(CFG, seed=seed, epsilon=0.3, noise=0.02, gamma=5.0)
    rng = np.random.default_rng(seed)
    for k in restart.REC2:  # histories too, with distinct values per array
        st[k] = st[k] + rng.standard_normal(st[k].shape)
    for k in restart.REC1:
        st[k] = rng.standard_normal(st[k].shape)
    return st


@pytest.mark.parametrize("nproc", [1, 2, 4])
def test_round_trip(tmp_path, nproc):
    st = state()
    paths = restart.write_restart(CFG, st, str(tmp_path), nproc=nproc)
    assert [os.path.basename(p) for p in paths] == [f"data00000002_instant.{r:03d}.dat" for r in range(nproc)]
    back = restart.read_restart(CFG, str(tmp_path), nproc=nproc)
    for k in restart.REC1 + restart.REC2:
        assert np.array_equal(back[k], st[k]), k
    assert not back["omegaxnp1"].any() and not back["omegaznp1"].any()


def test_fortran_record_layout(tmp_path):
    """Record bytes equal the Fortran column-major (0:nx,0:ny,0:nz) slabs,
    built independently from the (x, y, z)-indexed array, framed by 4-byte
    counts; the step variant of the name carries the step."""
    st = state(1)
    nproc, w = 2, CFG.nnx // 2
    restart.write_restart(CFG, st, str(tmp_path), nproc=nproc, istep=300000)
    nz1 = CFG.nnz + 1
    for r in range(nproc):
        raw = open(tmp_path / f"data00000002_instant.{r:03d}_00300000.dat", "rb").read()
        n1, n2 = 6 * 2 * nz1 * 8, 6 * w * CFG.nny * nz1 * 8
        assert len(raw) == 4 + n1 + 4 + 4 + n2 + 4
        marks = [raw[0:4], raw[4 + n1:8 + n1], raw[8 + n1:12 + n1], raw[-4:]]
        assert [int.from_bytes(m, "little") for m in marks] == [n1, n1, n2, n2]
        # record 1: (2, 0:nz) arrays, Fortran order = [re, im] per k
        rec1 = b"".join(np.asfortranarray(st[k].T).tobytes(order="F") for k in restart.REC1)
        assert raw[4:4 + n1] == rec1
        # record 2: F[x, y, z] = st[z, y, x], slab x in [r w, (r + 1) w)
        rec2 = b"".join(np.transpose(st[k], (2, 1, 0))[r * w:(r + 1) * w].tobytes(order="F")
                        for k in restart.REC2)
        assert raw[12 + n1:12 + n1 + n2] == rec2


def test_mean_arrays_come_from_rank_0(tmp_path):
    st = state(2)
    restart.write_restart(CFG, st, str(tmp_path), nproc=2)
    # change rank 1's mean record; the reader keeps rank 0's, as the reference
    p = tmp_path / "data00000002_instant.001.dat"
    raw = bytearray(open(p, "rb").read())
    raw[4:12] = np.float64(123.0).tobytes()
    open(p, "wb").write(bytes(raw))
    back = restart.read_restart(CFG, str(tmp_path), nproc=2)
    assert np.array_equal(back["clamb1n"], st["clamb1n"])


def test_rejects_bad_layouts(tmp_path):
    st = state()
    with pytest.raises(ValueError):
        restart.write_restart(CFG, st, str(tmp_path), nproc=3)   # 16 slots do not split in 3 pairs
    with pytest.raises(ValueError):
        restart.write_restart(CFG, st, str(tmp_path), nproc=8)   # nny / 2 = 4 not a multiple of 8
    restart.write_restart(CFG, st, str(tmp_path), nproc=2)
    with pytest.raises((ValueError, FileNotFoundError)):
        restart.read_restart(CFG, str(tmp_path), nproc=4)        # files of another split
    p = tmp_path / "data00000002_instant.000.dat"
    raw = open(p, "rb").read()
    open(p, "wb").write(raw[:-100])
    with pytest.raises(ValueError):
        restart.read_restart(CFG, str(tmp_path), nproc=2)        # truncated


@pytest.mark.parametrize("nproc", [1, 2, 4])
def test_velocity_dump_round_trip(tmp_path, nproc):
    """The 3Ddata dump: one record of ftmp(0:nx,0:ny,0:nz,1:3) per rank
    (Fortran order, i fastest), framed by 4-byte byte counts; the reader
    joins the streamwise slabs as post_poiseuilleflow.f90:63-70 does."""
    rng = np.random.default_rng(nproc)
    vel = rng.standard_normal((3, CFG.nnz + 1, CFG.nny, CFG.nnx))
    paths = restart.write_velocity_dump(CFG, vel, str(tmp_path), istep=1000, nproc=nproc)
    assert [os.path.basename(p) for p in paths] == [f"velocity00001000.{r:03d}.dat" for r in range(nproc)]
    w = CFG.nnx // nproc
    raw = np.fromfile(paths[-1], dtype=np.uint8)
    n = 3 * w * CFG.nny * (CFG.nnz + 1) * 8
    assert raw.size == n + 8
    assert int(raw[:4].view("<u4")[0]) == n and int(raw[-4:].view("<u4")[0]) == n
    # element (i, j, k, m) of the last rank's slab, Fortran order
    body = raw[4:-4].view("<f8").reshape(3, CFG.nnz + 1, CFG.nny, w)
    i, j, k, m = 1, 3, 5, 2
    assert body[m, k, j, i] == vel[m, k, j, (nproc - 1) * w + i]
    back = restart.read_velocity_dump(CFG, str(tmp_path), istep=1000, nproc=nproc)
    assert np.array_equal(back, vel)
