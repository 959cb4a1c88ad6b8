"""Extended-precision (numpy longdouble) dealiased Lamb vector for small
grids: every field is evaluated on the 3/2-padded x, y grid and the 2N-interval
Chebyshev grid with explicit DFT / cosine matrices, the products
H1 = oy w - re_p - oz v, H2 = oz u - ox w, H3 = ox v - oy u are formed
pointwise and transformed back and truncated exactly as getlamb does
(poiseuilleflow.f90:1625-1815, including the Nyquist slot of expand(-1)).
Test infrastructure: pins the oracle and the CUDA path against arithmetic
with 64-bit significands."""
import numpy as np

from channel_flow_gb300 import fields

LD = np.longdouble


def _mats(cfg):
    N, M = cfg.nnz, 2 * cfg.nnz
    PX, PY, KX, KY, NYQ = 3 * cfg.nnx // 2, 3 * cfg.nny // 2, cfg.nnx // 2, cfg.nny, cfg.nny // 2
    pi = LD(np.pi)
    # z: coefficients 0..N -> values at cos(pi p / M), p = 0..M; back: DCT-I, rows 0..N
    p = np.arange(M + 1, dtype=LD)
    n = np.arange(N + 1, dtype=LD)
    Tz = np.cos(pi * np.outer(p, n) / M)
    q = np.arange(M + 1, dtype=LD)
    w = np.ones(M + 1, dtype=LD)
    w[0] = w[-1] = LD(0.5)
    Wz = (LD(2) / M) * np.cos(pi * np.outer(n, q) / M) * w[None, :]
    Wz[0] *= LD(0.5)
    # y: slots -> padded wavenumbers
    ky_of_slot = np.array([j if j < NYQ else j - KY for j in range(KY)])
    ypts = np.arange(PY, dtype=LD)
    Ey = np.exp(1j * 2 * pi * np.outer(ypts, ky_of_slot.astype(LD)) / PY)   # [yp, slot]
    Ey[:, NYQ] = 0  # the Nyquist slot is zeroed before the transform
    # back: slots 0..NYQ from padded modes 0..NYQ, slots > NYQ from negative modes
    out_k = np.array([j if j <= NYQ else j - KY for j in range(KY)])
    Fy = np.exp(-1j * 2 * pi * np.outer(out_k.astype(LD), ypts) / PY) / PY   # [slot, yp]
    # x: half-complex kx = 0..KX-1 -> PX real points; back: kx = 0..KX-1
    xpts = np.arange(PX, dtype=LD)
    kx = np.arange(KX, dtype=LD)
    Ex = np.exp(1j * 2 * pi * np.outer(xpts, kx) / PX)                     # [xp, kx]
    Fx = np.exp(-1j * 2 * pi * np.outer(kx, xpts) / PX) / PX               # [kx, xp]
    return Tz, Wz, Ey, Fy, Ex, Fx


def _to_phys(a, mats):
    Tz, Wz, Ey, Fy, Ex, Fx = mats
    c = fields.as_complex(a).astype(np.clongdouble)         # [n][ky][kx]
    v = np.einsum("pn,nyx->pyx", Tz, c)                     # z values
    v = np.einsum("Yy,pyx->pYx", Ey, v)                     # y physical
    # x: real field from the half-complex modes; the x-mean keeps its real part
    v0 = v[:, :, 0].real
    rest = np.einsum("Xx,pYx->pYX", Ex[:, 1:], v[:, :, 1:])
    return v0[:, :, None] + 2 * rest.real                   # [p][yp][xp]


def _to_spec(f, mats):
    Tz, Wz, Ey, Fy, Ex, Fx = mats
    s = np.einsum("kX,pYX->pYk", Fx, f.astype(np.clongdouble))
    s = np.einsum("yY,pYk->pyk", Fy, s)
    s = np.einsum("np,pyk->nyk", Wz, s)
    out = np.empty(s.shape[:2] + (2 * s.shape[2],))
    out[:, :, 0::2] = np.asarray(s.real, dtype=np.float64)
    out[:, :, 1::2] = np.asarray(s.imag, dtype=np.float64)
    return out


def lamb(cfg, st):
    mats = _mats(cfg)
    P = {k: _to_phys(st[k], mats) for k in ("unp1", "vnp1", "wnp1", "omegaxnp1", "omegaynp1", "omegaznp1")}
    u, v, w = P["unp1"], P["vnp1"], P["wnp1"]
    ox, oy, oz = P["omegaxnp1"], P["omegaynp1"], P["omegaznp1"]
    h1 = (oy * w - LD(cfg.re_p)) - oz * v
    h2 = oz * u - ox * w
    h3 = ox * v - oy * u
    return _to_spec(h1, mats), _to_spec(h2, mats), _to_spec(h3, mats)


def _to_spec_ld(f, mats):
    """_to_spec without the final rounding: clongdouble [n][ky][kx]."""
    Tz, Wz, Ey, Fy, Ex, Fx = mats
    s = np.einsum("kX,pYX->pYk", Fx, f.astype(np.clongdouble))
    s = np.einsum("yY,pYk->pyk", Fy, s)
    return np.einsum("np,pyk->nyk", Wz, s)


def nonlinear_histories(cfg, st):
    """rhsvn and rhsomegayn as getnonlinear leaves them (poiseuilleflow.f90:
    1502-1609): h_v = k^2 H2 + i a D H1 + i b D H3 and h_g = i a H3 - i b H1
    (D the Chebyshev derivative of dz, :570-599), as values at the Gauss-
    Lobatto points cos(pi k / N), all in longdouble from the products on;
    rounded to FP64 once, in the field layout [n][ky][2 kx]."""
    mats = _mats(cfg)
    P = {k: _to_phys(st[k], mats) for k in ("unp1", "vnp1", "wnp1", "omegaxnp1", "omegaynp1", "omegaznp1")}
    u, v, w = P["unp1"], P["vnp1"], P["wnp1"]
    ox, oy, oz = P["omegaxnp1"], P["omegaynp1"], P["omegaznp1"]
    h1 = _to_spec_ld((oy * w - LD(cfg.re_p)) - oz * v, mats)
    h2 = _to_spec_ld(oz * u - ox * w, mats)
    h3 = _to_spec_ld(ox * v - oy * u, mats)
    N = cfg.nnz
    D = np.zeros((N + 1, N + 1), dtype=LD)
    for i in range(N):
        for j in range(i + 1, N + 1):
            if (i + j) % 2:
                D[i, j] = LD(j) if i == 0 else LD(2 * j)
    ia, ib = fields.wavenumbers(cfg)
    a = np.asarray(ia, dtype=LD)[None, None, :]
    b = np.asarray(ib, dtype=LD)[None, :, None]
    k2 = a * a + b * b
    d1 = np.einsum("ij,jyx->iyx", D, h1)
    d3 = np.einsum("ij,jyx->iyx", D, h3)
    hv = k2 * h2 + 1j * a * d1 + 1j * b * d3
    hg = 1j * a * h3 - 1j * b * h1
    n = np.arange(N + 1, dtype=LD)
    G = np.cos(LD(np.pi) * np.outer(n, n) / N)  # [k][j]: T_j at cos(pi k / N)
    out = []
    for h in (hv, hg):
        g = np.einsum("kj,jyx->kyx", G, h)
        o = np.empty(g.shape[:2] + (2 * g.shape[2],))
        o[:, :, 0::2] = np.asarray(g.real, dtype=np.float64)
        o[:, :, 1::2] = np.asarray(g.imag, dtype=np.float64)
        out.append(o)
    return out[0], out[1]
