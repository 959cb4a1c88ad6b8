"""Statistics the way the reference forms them (statistics,
poiseuilleflow.f90:2666-3198): u, v, w transformed to the physical
nnx x nny x (nz+1) grid, then plane means, covariances and the energy sum
over grid points.  NumPy, test-only."""
import numpy as np

from channel_flow_gb300 import fields


def physical(cfg, a):
    """(nnz+1, nny, nnx) spectral array -> physical values on the GL x grid:
    u(x, y, z_k) = sum over the full spectrum of u^ e^{i(kx x + ky y)}."""
    n = cfg.nnz
    c = fields.as_complex(a).copy()
    c[:, cfg.nny // 2, :] = 0.0
    T0 = np.cos(np.pi * np.outer(np.arange(n + 1), np.arange(n + 1)) / n)
    g = np.tensordot(T0, c, axes=(1, 0))
    full = np.zeros(g.shape[:2] + (cfg.nnx // 2 + 1,), complex)
    full[:, :, :cfg.kx] = g
    return np.fft.irfft(np.fft.ifft(full, axis=1) * cfg.nny, n=cfg.nnx, axis=2) * cfg.nnx


def statistics(cfg, st):
    u, v, w = (physical(cfg, st[k]) for k in ("unp1", "vnp1", "wnp1"))
    n = cfg.nnz
    z = np.cos(np.pi * np.arange(n + 1) / n)
    mean = lambda f: f.mean(axis=(1, 2))
    ua, va, wa = mean(u), mean(v), mean(w)
    up, vp, wp = u - ua[:, None, None], v - va[:, None, None], w - wa[:, None, None]
    out = {"z": z, "u": ua, "v": va, "w": wa, "uu": mean(up * up), "vv": mean(vp * vp), "ww": mean(wp * wp),
           "uv": mean(up * vp), "uw": mean(up * wp), "vw": mean(vp * wp),
           "energy": 0.5 * float(np.sum(u * u + v * v + w * w))}
    # d<u>/dz at the walls from the Chebyshev coefficients of <u>
    coef = fields._dct1_matrix(n) @ ua
    dcoef = fields.cheb_derivative_matrix(n) @ coef
    top, bot = float(np.sum(dcoef)), float(np.sum(dcoef * (-1.0) ** np.arange(n + 1)))
    out["u_tau_top"], out["u_tau_bottom"] = np.sqrt(abs(top) / cfg.re), np.sqrt(abs(bot) / cfg.re)
    out["re_centre"] = ua[n // 2] * cfg.re
    ub = sum(ua[k] * abs(z[k + 1] - z[k]) for k in range(n // 2, n))
    out["re_bulk"] = 2.0 * ub * cfg.re
    return out
