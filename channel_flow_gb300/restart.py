"""Restart files in the reference's layout, on the host (NumPy).

The reference writes one Fortran unformatted sequential file per MPI rank in
``output`` (poiseuilleflow.f90:2460-2504) and reads it in ``initial``
(poiseuilleflow.f90:1873-1917).  Each file has two records, each framed by
4-byte little-endian byte counts:

* record 1: clamb1n, clamb1nm1, clamb3n, clamb3nm1, au0, w0, each (2, 0:nz);
* record 2: vnp1, omegaynp1, rhsvn, rhsomegayn, unp1, wnp1, each
  (0:nx, 0:ny, 0:nz) for the rank's streamwise slab of nx + 1 = nnx / nproc
  interleaved (re, im) slots, starting at slot rank * (nx + 1).

This module reads and writes those files for any nproc: it splits a one-rank
state into nproc slabs, or joins nproc files into one state.
``Channel.write_restart`` / ``Channel.read_restart`` do the same in the CUDA
library (chf_write_restart / chf_read_restart), straight from and to device
memory.
"""
import os

import numpy as np

from .config import ChannelConfig
from .fields import empty_state

REC1 = ("clamb1n", "clamb1nm1", "clamb3n", "clamb3nm1", "au0", "w0")
REC2 = ("vnp1", "omegaynp1", "rhsvn", "rhsomegayn", "unp1", "wnp1")
_MARK = np.dtype("<u4")


def file_name(rank: int, tag: int = 2, istep: int = -1) -> str:
    """Format 2111 ('data', i8.8, '_instant.', i3.3, '.dat') or, with a step,
    format 22211 (adds '_', i8.8)."""
    if istep >= 0:
        return f"data{tag:08d}_instant.{rank:03d}_{istep:08d}.dat"
    return f"data{tag:08d}_instant.{rank:03d}.dat"


def check_nproc(cfg: ChannelConfig, nproc: int) -> int:
    """Slots per rank; the reference's own constraints (paraandcons.f90:4-8)."""
    if nproc < 1 or cfg.nnx % (2 * nproc) or (cfg.nny // 2) % nproc:
        raise ValueError("nnx must be a multiple of 2 nproc and nny / 2 a multiple of nproc")
    w = cfg.nnx // nproc
    if 6 * w * cfg.nny * (cfg.nnz + 1) * 8 > 0x7FFFFFF0:
        raise ValueError("a record above 2 GiB needs more ranks")
    return w


def _write_record(f, arrays):
    nbytes = sum(a.nbytes for a in arrays)
    np.array([nbytes], dtype=_MARK).tofile(f)
    for a in arrays:
        np.ascontiguousarray(a, dtype="<f8").tofile(f)
    np.array([nbytes], dtype=_MARK).tofile(f)


def _read_record(f, nbytes, what):
    head = np.fromfile(f, dtype=_MARK, count=1)
    if head.size != 1 or int(head[0]) != nbytes:
        raise ValueError(f"{what}: record of {nbytes} bytes expected")
    data = np.fromfile(f, dtype="<f8", count=nbytes // 8)
    tail = np.fromfile(f, dtype=_MARK, count=1)
    if data.size != nbytes // 8 or tail.size != 1 or int(tail[0]) != nbytes:
        raise ValueError(f"{what}: truncated or corrupt record")
    return data


def write_restart(cfg: ChannelConfig, st: dict, directory: str, nproc: int = 1, tag: int = 2,
                  istep: int = -1) -> list:
    """Write st (a one-rank state dict, fields.FIELD_NAMES + MEAN_NAMES) as
    nproc rank files; returns their paths."""
    w = check_nproc(cfg, nproc)
    paths = []
    for r in range(nproc):
        p = os.path.join(directory, file_name(r, tag, istep))
        with open(p, "wb") as f:
            _write_record(f, [st[k] for k in REC1])
            _write_record(f, [st[k][:, :, r * w:(r + 1) * w] for k in REC2])
        paths.append(p)
    return paths


def read_restart(cfg: ChannelConfig, directory: str, nproc: int = 1, tag: int = 2,
                 istep: int = -1) -> dict:
    """Join nproc rank files into one state dict.  omegaxnp1 / omegaznp1 are
    not in the files and come back as zeros (the solve recomputes them);
    the mean arrays are rank 0's, the ones the reference uses."""
    w = check_nproc(cfg, nproc)
    st = empty_state(cfg)
    nz1 = cfg.nnz + 1
    n1, n2 = 6 * 2 * nz1 * 8, 6 * w * cfg.nny * nz1 * 8
    for r in range(nproc):
        p = os.path.join(directory, file_name(r, tag, istep))
        with open(p, "rb") as f:
            m = _read_record(f, n1, p).reshape(6, nz1, 2)
            d = _read_record(f, n2, p).reshape(6, nz1, cfg.nny, w)
        if r == 0:
            for i, k in enumerate(REC1):
                st[k][...] = m[i]
        for i, k in enumerate(REC2):
            st[k][:, :, r * w:(r + 1) * w] = d[i]
    return st


# ---------------------------------------------------------------------------
# The 3Ddata velocity dump of statistics (poiseuilleflow.f90:2745-2764):
# one file per rank, one record ftmp(0:nx, 0:ny, 0:nz, 1:3) of the rank's
# streamwise slab of nnx / nproc physical points (u + u0, w, v), read and
# joined by post-processing/post_poiseuilleflow.f90:63-70.
# ---------------------------------------------------------------------------
def velocity_file_name(istep: int, rank: int) -> str:
    """Format 212 of statistics: 'velocity', i8.8, '.', i3.3, '.dat'."""
    return f"velocity{istep:08d}.{rank:03d}.dat"


def write_velocity_dump(cfg: ChannelConfig, vel: np.ndarray, directory: str, istep: int = 0,
                        nproc: int = 1) -> list:
    """Write vel (3, nz+1, nny, nnx) = (u + u0, w, v) on the physical grid as
    nproc rank files; returns their paths."""
    w = check_nproc(cfg, nproc)
    paths = []
    for r in range(nproc):
        p = os.path.join(directory, velocity_file_name(istep, r))
        with open(p, "wb") as f:
            _write_record(f, [vel[:, :, :, r * w:(r + 1) * w]])
        paths.append(p)
    return paths


def read_velocity_dump(cfg: ChannelConfig, directory: str, istep: int = 0, nproc: int = 1) -> np.ndarray:
    """Join nproc rank files of the velocity dump into (3, nz+1, nny, nnx),
    the array ftmp2 that post_poiseuilleflow.f90:63-70 assembles."""
    w = check_nproc(cfg, nproc)
    nz1 = cfg.nnz + 1
    out = np.zeros((3, nz1, cfg.nny, cfg.nnx))
    n = 3 * w * cfg.nny * nz1 * 8
    for r in range(nproc):
        p = os.path.join(directory, velocity_file_name(istep, r))
        with open(p, "rb") as f:
            d = _read_record(f, n, p).reshape(3, nz1, cfg.nny, w)
            if f.read(1):
                raise ValueError(f"{p}: data after the record")
        out[:, :, :, r * w:(r + 1) * w] = d
    return out
