"""Seeded initial fields and host-side spectral helpers (NumPy).

The reference initialises with an unseeded Fortran ``random_number``
(poiseuilleflow.f90:2121-2171), so its initial state cannot be reproduced.
This module builds the same kind of state from a seeded counter-based
generator (NumPy Philox) so that every run, on any host, starts from the same
bits.  It is host-side set-up, like the reference's ``initial``/``input``
(poiseuilleflow.f90:1824-1980, 2086-2339); the time step itself runs in the
CUDA library.

State dictionaries use the reference's module arrays (paraandcons.f90:28-38):
spectral fields as float64 arrays of shape (nnz+1, nny, nnx) (C order) which
is the Fortran (0:nx,0:ny,0:nz) layout, and mean-mode arrays of shape
(nnz+1, 2) which is the Fortran (2,0:nz) layout.
"""
import numpy as np

from .config import ChannelConfig

FIELD_NAMES = ("vnp1", "omegaynp1", "unp1", "wnp1", "omegaxnp1", "omegaznp1", "rhsvn", "rhsomegayn")
MEAN_NAMES = ("clamb1n", "clamb1nm1", "clamb3n", "clamb3nm1", "au0", "w0")


def wavenumbers(cfg: ChannelConfig):
    """iapha(0:nhx), ibeta(0:ny) as at poiseuilleflow.f90:123-134 (one rank)."""
    ny = cfg.nny - 1
    ibeta = np.zeros(cfg.nny)
    for j in range(0, (ny + 1) // 2 + 1):
        ibeta[j] = j / cfg.beta
        if j <= (ny - 1) // 2 - 1:
            ibeta[ny - j] = (-j - 1) / cfg.beta
    iapha = np.arange(cfg.kx, dtype=np.float64) / cfg.aphi
    return iapha, ibeta


def zpoints(n: int) -> np.ndarray:
    return np.cos(np.pi * np.arange(n + 1) / n)


def cheb_derivative_matrix(n: int) -> np.ndarray:
    """Matrix of dz (poiseuilleflow.f90:570-599) acting on coefficients."""
    D = np.zeros((n + 1, n + 1))
    for i in range(n):
        for j in range(i + 1, n + 1):
            if (i + j) % 2:
                D[i, j] = j if i == 0 else 2.0 * j
    return D


def _dct1_matrix(n: int) -> np.ndarray:
    """Values at z_k -> Chebyshev coefficients (the 'transform(-1)' z part)."""
    k = np.arange(n + 1)
    C = np.cos(np.pi * np.outer(k, k) / n)
    w = np.ones(n + 1)
    w[0] = w[-1] = 0.5
    M = (2.0 / n) * C * w[None, :]
    M[0] *= 0.5
    M[-1] *= 0.5
    return M


def phys_to_spec(cfg: ChannelConfig, f: np.ndarray) -> np.ndarray:
    """Physical (nnz+1, nny, nnx) -> spectral, as transform(-1) at
    poiseuilleflow.f90:967-1003: Chebyshev in z, then x forward FFT keeping
    kx = 0..nnx/2-1, y forward FFT, normalised by 1/(nnx*nny)."""
    c = np.tensordot(_dct1_matrix(cfg.nnz), f, axes=(1, 0))
    fx = np.fft.fft(c, axis=2)[:, :, : cfg.kx]
    fxy = np.fft.fft(fx, axis=1) / (cfg.nnx * cfg.nny)
    out = np.empty(f.shape)
    out[:, :, 0::2] = fxy.real
    out[:, :, 1::2] = fxy.imag
    return out


def as_complex(a: np.ndarray) -> np.ndarray:
    return a.view(np.complex128)


def recover_velocity(cfg: ChannelConfig, st: dict, modes="all") -> None:
    """u, w, omega_x, omega_z from v and omega_y for every mode with k^2 != 0,
    as getvelocityandvorticity (poiseuilleflow.f90:2347-2407)."""
    iapha, ibeta = wavenumbers(cfg)
    D = cheb_derivative_matrix(cfg.nnz)
    v = as_complex(st["vnp1"])
    oy = as_complex(st["omegaynp1"])
    u = as_complex(st["unp1"])
    w = as_complex(st["wnp1"])
    ox = as_complex(st["omegaxnp1"])
    oz = as_complex(st["omegaznp1"])
    a = iapha[None, None, :]
    b = ibeta[None, :, None]
    k2 = a * a + b * b
    mask = np.broadcast_to(k2 != 0.0, v.shape)
    k2s = np.where(k2 == 0.0, 1.0, k2)
    dv = np.tensordot(D, v, axes=(1, 0))
    un = (1j * a * dv - 1j * b * oy) / k2s
    wn = (1j * b * dv + 1j * a * oy) / k2s
    u[mask] = un[mask]
    w[mask] = wn[mask]
    dw = np.tensordot(D, w, axes=(1, 0))
    du = np.tensordot(D, u, axes=(1, 0))
    oxn = dw - 1j * b * v
    ozn = -du + 1j * a * v
    ox[mask] = oxn[mask]
    oz[mask] = ozn[mask]


def empty_state(cfg: ChannelConfig) -> dict:
    shape = (cfg.nnz + 1, cfg.nny, cfg.nnx)
    st = {k: np.zeros(shape) for k in FIELD_NAMES}
    st.update({k: np.zeros((cfg.nnz + 1, 2)) for k in MEAN_NAMES})
    return st


def _set_mean(cfg: ChannelConfig, st: dict) -> None:
    """au0/w0 from the (0,0) modes of u and w (poiseuilleflow.f90:1937-1943)."""
    st["au0"][:, 0] = st["unp1"][:, 0, 0]
    st["au0"][:, 1] = st["unp1"][:, 0, 1]
    st["w0"][:, 0] = st["wnp1"][:, 0, 0]
    st["w0"][:, 1] = st["wnp1"][:, 0, 1]


def reference_like_state(cfg: ChannelConfig, seed: int = 0, epsilon: float = 1.0,
                         noise: float = 0.1, gamma: float = 10.0) -> dict:
    """The analytic-plus-noise field of ``input`` (poiseuilleflow.f90:2086-2339)
    with a seeded generator: v, omega_y, u, w get the reference's analytic
    perturbation of amplitude ``epsilon`` plus uniform noise in [-noise, noise]
    at every grid point (walls set to 0); the laminar profile gamma*(1-z^2) is
    added to the (0,0) mode of u and gamma*2z (walls zeroed, as the reference
    does) to omega_z.  Histories are zero, as after ``input``."""
    rng = np.random.Generator(np.random.Philox(seed))
    pi = np.pi
    lx = 2 * pi * cfg.aphi
    ly = 2 * pi * cfg.beta
    x = 2 * pi * np.arange(cfg.nnx) / cfg.nnx * cfg.aphi
    y = 2 * pi * np.arange(cfg.nny) / cfg.nny * cfg.beta
    z = zpoints(cfg.nnz)
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    sx1, sx2 = np.sin(2 * pi * X / lx), np.sin(4 * pi * X / lx)
    cx1, cx2 = np.cos(2 * pi * X / lx), np.cos(4 * pi * X / lx)
    sy1, sy2 = np.sin(2 * pi * Y / ly), np.sin(4 * pi * Y / ly)
    cy1, cy2 = np.cos(2 * pi * Y / ly), np.cos(4 * pi * Y / ly)
    e = epsilon

    def nz():
        return noise * (2.0 * rng.random(Z.shape) - 1.0)

    v = -e * (1.0 + np.cos(pi * Z)) * (sx1 * sy1 + sx2 * sy1 + sx1 * sy2) + nz()
    oy = e * 2.0 * pi * np.sin(pi * Z) * (
        lx / ly * (cx1 * cy1 + 0.5 * cx2 * cy1 + 2.0 * cx1 * cy2)
        + ly / lx * (0.5 * cx1 * cy1 + cx2 * cy1 + 0.25 * cx1 * cy2)) + nz()
    u = e * lx * np.sin(pi * Z) * (cx1 * sy1 + 0.5 * cx2 * sy1 + cx1 * sy2) + nz()
    w = -e * ly * np.sin(pi * Z) * (0.5 * sx1 * cy1 + 0.5 * sx2 * cy1 + 0.25 * sx1 * cy2) + nz()
    for a in (v, oy, u, w):
        a[0] = 0.0
        a[-1] = 0.0
    st = empty_state(cfg)
    st["vnp1"] = phys_to_spec(cfg, v)
    st["omegaynp1"] = phys_to_spec(cfg, oy)
    st["unp1"] = phys_to_spec(cfg, u)
    st["wnp1"] = phys_to_spec(cfg, w)
    recover_velocity(cfg, st)
    lam_u = np.broadcast_to((gamma * (1.0 - z * z))[:, None, None], Z.shape).copy()
    lam_o = np.broadcast_to((gamma * 2.0 * z)[:, None, None], Z.shape).copy()
    for a in (lam_u, lam_o):
        a[0] = 0.0
        a[-1] = 0.0
    st["unp1"] += phys_to_spec(cfg, lam_u)
    st["omegaznp1"] += phys_to_spec(cfg, lam_o)
    _set_mean(cfg, st)
    return st


def bulk_velocity(st: dict) -> float:
    """U_b = (1/2) int_{-1}^{1} u dz of the mean profile au0 (Chebyshev
    coefficients): sum over even n of au0_n / (1 - n^2)."""
    a = st["au0"][:, 0]
    n = np.arange(a.size)
    even = n % 2 == 0
    return float(np.sum(a[even] / (1.0 - n[even] ** 2.0)))


def laminar_state(cfg: ChannelConfig, gamma: float = None) -> dict:
    """Plane Poiseuille flow U = gamma (1 - z^2) alone in the (0,0) mode, with
    omega_z = -dU/dz = 2 gamma z.  With gamma = re*re_p/2 and steady mean
    histories (clamb1n = clamb1nm1 = -re_p) it is a fixed point of the step."""
    if gamma is None:
        gamma = cfg.re * cfg.re_p / 2.0
    st = empty_state(cfg)
    n = cfg.nnz
    cu = np.zeros(n + 1)
    cu[0] = 0.5 * gamma
    cu[2] = -0.5 * gamma
    co = np.zeros(n + 1)
    co[1] = 2.0 * gamma
    st["unp1"][:, 0, 0] = cu
    st["omegaznp1"][:, 0, 0] = co
    _set_mean(cfg, st)
    st["clamb1n"][:, 0] = -cfg.re_p
    st["clamb1nm1"][:, 0] = -cfg.re_p
    return st


def lowmode_state(cfg: ChannelConfig, seed: int = 0, amp: float = 1e-3, nmodes: int = 4,
                  gamma: float = 1.0) -> dict:
    """Laminar gamma (1 - z^2) plus a seeded divergence-free perturbation of
    amplitude ``amp`` in streamwise modes 0..nmodes-1 and spanwise modes
    |ky| < nmodes.  v carries the factor (1 - z^2)^2 and omega_y the factor
    (1 - z^2), so both satisfy the wall conditions; u, w, omega_x, omega_z
    follow from getvelocityandvorticity."""
    rng = np.random.Generator(np.random.Philox(seed))
    st = empty_state(cfg)
    n = cfg.nnz
    z = zpoints(n)
    v = as_complex(st["vnp1"])
    oy = as_complex(st["omegaynp1"])
    M = _dct1_matrix(n)
    deg = min(6, n - 4)
    for i in range(min(nmodes, cfg.kx)):
        for jj in range(-(nmodes - 1), nmodes):
            if i == 0 and jj == 0:
                continue
            if abs(jj) >= cfg.nny // 2:
                continue
            j = jj % cfg.nny
            pv = np.polynomial.chebyshev.chebval(z, rng.standard_normal(deg + 1) + 1j * rng.standard_normal(deg + 1))
            po = np.polynomial.chebyshev.chebval(z, rng.standard_normal(deg + 1) + 1j * rng.standard_normal(deg + 1))
            v[:, j, i] = M @ (amp * (1.0 - z * z) ** 2 * pv)
            oy[:, j, i] = M @ (amp * (1.0 - z * z) * po)
    # a real field: kx = 0 modes satisfy f(-ky) = conj f(ky)
    for jj in range(1, nmodes):
        if jj < cfg.nny // 2:
            v[:, (-jj) % cfg.nny, 0] = np.conj(v[:, jj, 0])
            oy[:, (-jj) % cfg.nny, 0] = np.conj(oy[:, jj, 0])
    recover_velocity(cfg, st)
    st["unp1"][:, 0, :2] = 0.0
    st["omegaznp1"][:, 0, :2] = 0.0
    st["unp1"][0, 0, 0] = 0.5 * gamma
    st["unp1"][2, 0, 0] = -0.5 * gamma
    st["omegaznp1"][1, 0, 0] = 2.0 * gamma
    _set_mean(cfg, st)
    return st


def _cheb_values_matrix(n: int) -> np.ndarray:
    k = np.arange(n + 1)
    return np.cos(np.pi * np.outer(k, k) / n)  # [point, coefficient]


def loglaw_profile(z: np.ndarray, re_tau: float, u_tau: float = 1.0) -> np.ndarray:
    """Turbulent mean velocity at the points z: Reichardt's wall law
    u+ = ln(1 + k y+) / k + 7.8 (1 - exp(-y+/11) - (y+/11) exp(-y+/3)),
    k = 0.41, y+ = (1 - |z|) Re_tau (the viscous sublayer, buffer layer and
    log layer in one smooth formula), times u_tau."""
    yp = (1.0 - np.abs(z)) * re_tau
    k = 0.41
    return u_tau * (np.log1p(k * yp) / k + 7.8 * (1.0 - np.exp(-yp / 11.0) - (yp / 11.0) * np.exp(-yp / 3.0)))


def turbulent_start_state(cfg: ChannelConfig, seed: int = 0, u_centre: float = None,
                          frac: float = 0.1, mode_frac: float = 0.25, deg_frac: float = 0.25,
                          loglaw: bool = False) -> dict:
    """Laminar profile u_centre (1 - z^2) (or, with ``loglaw``, the wall-law
    mean profile of loglaw_profile at Re_tau = re sqrt(re_p)) plus a seeded
    divergence-free perturbation whose rms velocity is ``frac * u_centre``.

    The perturbation lives in the lowest ``mode_frac`` of the streamwise and
    spanwise modes; its wall-normal profiles are (1 - z^2)^2 P(z) for v and
    (1 - z^2) Q(z) for omega_y with random Chebyshev series P, Q of degree
    ``deg_frac * nnz`` (decaying spectrum), so every wall condition holds;
    u, w, omega_x, omega_z follow from getvelocityandvorticity.  The default
    u_centre is the laminar centreline re*re_p/2 when that is O(1) (channels
    scaled by the laminar centreline speed) and otherwise the turbulent
    centreline 2.5 ln(Re_tau) + 5.5 in wall units (u_tau = sqrt(re_p))."""
    rng = np.random.Generator(np.random.Philox(seed))
    n = cfg.nnz
    z = zpoints(n)
    mean_vals = None
    if loglaw:
        mean_vals = loglaw_profile(z, cfg.re * np.sqrt(cfg.re_p), np.sqrt(cfg.re_p))
        u_centre = float(mean_vals[n // 2])
    if u_centre is None:
        lam = cfg.re * cfg.re_p / 2.0
        if lam <= 2.0:
            u_centre = lam
        else:
            re_tau = cfg.re * np.sqrt(cfg.re_p)
            u_centre = 2.5 * np.log(re_tau) + 5.5
    st = empty_state(cfg)
    M = _dct1_matrix(n)
    deg = max(2, min(int(deg_frac * n), n - 4))
    nkx = max(1, int(mode_frac * cfg.kx))
    nky = max(1, int(mode_frac * cfg.nny / 2))
    v = as_complex(st["vnp1"])
    oy = as_complex(st["omegaynp1"])
    damp = np.exp(-np.arange(deg + 1) / max(1.0, deg / 3.0))
    wv = (1.0 - z * z) ** 2
    wo = 1.0 - z * z
    for i in range(nkx):
        for jj in range(-(nky - 1), nky):
            if i == 0 and jj <= 0:
                continue  # kx = 0: fill jj > 0, mirror below
            j = jj % cfg.nny
            cv = (rng.standard_normal(deg + 1) + 1j * rng.standard_normal(deg + 1)) * damp
            co = (rng.standard_normal(deg + 1) + 1j * rng.standard_normal(deg + 1)) * damp
            v[:, j, i] = M @ (wv * np.polynomial.chebyshev.chebval(z, cv))
            oy[:, j, i] = M @ (wo * np.polynomial.chebyshev.chebval(z, co))
    for jj in range(1, nky):
        v[:, (-jj) % cfg.nny, 0] = np.conj(v[:, jj, 0])
        oy[:, (-jj) % cfg.nny, 0] = np.conj(oy[:, jj, 0])
    recover_velocity(cfg, st)
    # physical mean square of the perturbation velocity (Parseval in x, y;
    # kx > 0 modes stand for their conjugate partners too)
    T = _cheb_values_matrix(n)
    ms = 0.0
    for name in ("unp1", "vnp1", "wnp1"):
        vals = np.tensordot(T, as_complex(st[name]), axes=(1, 0))
        p = np.abs(vals) ** 2
        p[:, :, 1:] *= 2.0
        ms += p.sum(axis=(1, 2)).mean()
    scale = frac * u_centre / np.sqrt(ms / 3.0) if ms > 0 else 0.0
    for name in ("vnp1", "omegaynp1", "unp1", "wnp1", "omegaxnp1", "omegaznp1"):
        st[name] *= scale
    st["unp1"][:, 0, :2] = 0.0
    st["omegaznp1"][:, 0, :2] = 0.0
    if mean_vals is None:
        st["unp1"][0, 0, 0] = 0.5 * u_centre
        st["unp1"][2, 0, 0] = -0.5 * u_centre
        st["omegaznp1"][1, 0, 0] = 2.0 * u_centre
    else:  # Chebyshev coefficients of the wall-law profile; omega_z = -dU/dz
        cu = M @ mean_vals
        st["unp1"][:, 0, 0] = cu
        st["omegaznp1"][:, 0, 0] = -(cheb_derivative_matrix(n) @ cu)
    _set_mean(cfg, st)
    return st


def collocation_matrices(n: int):
    """T0, T2, T4 at the Gauss-Lobatto points (the SCHEB matrices,
    poiseuilleflow.f90:3272-3342), from exact Chebyshev calculus."""
    T0 = _cheb_values_matrix(n)
    D = cheb_derivative_matrix(n)
    D2 = D @ D
    return T0, T0 @ D2, T0 @ D2 @ D2


def orr_sommerfeld_mode(cfg: ChannelConfig, kx: int = 1, U=None):
    """Least-stable Orr-Sommerfeld eigenpair of v about U(z) (default
    U = 1 - z^2) for streamwise mode kx (alpha = kx/aphi, beta = 0), in the
    reference's collocation discretisation: the equation
        d/dt (D^2 - a^2) v = -i a U (D^2 - a^2) v + i a U'' v + (1/re) (D^2 - a^2)^2 v
    at the interior points 2..N-2 plus the four wall conditions v = v' = 0
    (the rows of get_coef_v, poiseuilleflow.f90:3348-3381).  Returns
    (sigma, coefficients): v(t) ~ exp(sigma t)."""
    import scipy.linalg
    n = cfg.nnz
    a = kx / cfg.aphi
    z = zpoints(n)
    T0, T2, T4 = collocation_matrices(n)
    if U is None:
        Uz, Upp = 1.0 - z * z, -2.0 * np.ones_like(z)
    else:
        Uz, Upp = U
    rows = np.arange(2, n - 1)
    lap = T2[rows] - a * a * T0[rows]
    bih = T4[rows] - 2 * a * a * T2[rows] + a ** 4 * T0[rows]
    Lmat = np.zeros((n + 1, n + 1), dtype=complex)
    Mmat = np.zeros((n + 1, n + 1), dtype=complex)
    j = np.arange(n + 1)
    Lmat[0] = 1.0
    Lmat[1] = (-1.0) ** j
    Lmat[2] = j ** 2
    Lmat[3] = -((-1.0) ** j) * j ** 2
    Lmat[4:] = -1j * a * Uz[rows, None] * lap + 1j * a * Upp[rows, None] * T0[rows] + bih / cfg.re
    Mmat[4:] = lap
    w, V = scipy.linalg.eig(Lmat, Mmat)
    ok = np.isfinite(w)
    w, V = w[ok], V[:, ok]
    i = int(np.argmax(w.real))
    return w[i], V[:, i]


def orr_sommerfeld_state(cfg: ChannelConfig, amp: float = 1e-6, kx: int = 1) -> dict:
    """Laminar Poiseuille flow U = 1 - z^2 (with steady mean histories) plus
    the least-stable two-dimensional Orr-Sommerfeld mode of streamwise mode kx
    at amplitude amp (max |v| coefficient); u, omega_z follow from
    getvelocityandvorticity (omega_y = w = 0 for a 2D mode)."""
    sigma, vec = orr_sommerfeld_mode(cfg, kx)
    st = laminar_state(cfg, gamma=1.0)  # the fixed point needs re * re_p = 2
    vec = vec / np.abs(vec).max() * amp
    v = as_complex(st["vnp1"])
    v[:, 0, kx] = vec
    recover_velocity(cfg, st)  # k^2 != 0 modes only: the (0,0) mode stays laminar
    return st
