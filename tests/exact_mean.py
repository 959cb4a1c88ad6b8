"""Extended-precision (numpy longdouble) value of the (0,0) Fourier mode of a
dealiased product, by Parseval: sum over modes k of f_k g_{-k}, with exact
Chebyshev products T_m T_n = (T_{m+n} + T_{|m-n|})/2 truncated to degree N.
Test infrastructure: an independent check of how accurately an
implementation forms the mean Lamb vector (REF:1482-1487)."""
import numpy as np

from channel_flow_gb300 import fields


def _cheb_prod_trunc(a, b, N):
    out = np.zeros(a.shape[:-1] + (N + 1,), dtype=a.dtype)
    n = np.arange(N + 1)
    for m in range(N + 1):
        prod = a[..., m:m + 1] * b * 0.5
        s = m + n
        keep = s <= N
        out[..., s[keep]] += prod[..., keep]
        d = np.abs(m - n)
        # several q can map to the same |m - q|; accumulate one at a time
        for q in range(N + 1):
            out[..., d[q]] += prod[..., q]
    return out


def mean_product(cfg, f, g):
    N, NYQ = cfg.nnz, cfg.nny // 2
    F = np.moveaxis(fields.as_complex(f).astype(np.clongdouble), 0, -1).copy()
    G = np.moveaxis(fields.as_complex(g).astype(np.clongdouble), 0, -1).copy()
    F[NYQ] = 0
    G[NYQ] = 0
    kyn = (-np.arange(cfg.nny)) % cfg.nny
    # kx = 0: the imaginary part of the streamwise mean is dropped by the c2r
    F0 = 0.5 * (F[:, 0, :] + np.conj(F[kyn, 0, :]))
    G0 = 0.5 * (G[:, 0, :] + np.conj(G[kyn, 0, :]))
    tot = _cheb_prod_trunc(F0, G0[kyn], N).sum(axis=0)
    Fp, Gp = F[:, 1:, :], G[:, 1:, :]
    tot += _cheb_prod_trunc(Fp, np.conj(Gp), N).sum(axis=(0, 1))
    tot += _cheb_prod_trunc(np.conj(Fp), Gp, N).sum(axis=(0, 1))
    return tot


def mean_h1(cfg, st):
    """H1(0,0) = <omega_y w> - <omega_z v> - re_p, Chebyshev coefficients."""
    h = mean_product(cfg, st["omegaynp1"], st["wnp1"]) - mean_product(cfg, st["omegaznp1"], st["vnp1"])
    h[0] -= cfg.re_p
    return np.array(h, dtype=np.complex128)
