"""Channel configuration, mirroring the compile-time parameters of
paraandcons.f90:4-25 (nnx, nny, nnz, aphi, beta, dt, re, re_p) for one rank.

Axis names follow the reference: x streamwise (Fourier, half-complex),
y spanwise (Fourier, full complex), z wall-normal (Chebyshev, points
z_k = cos(pi k / nz), poiseuilleflow.f90:146-148).  A grid quoted as
"Nx x Ny(wall) x Nz(span)" = nnx x (nnz+1) x nny.
"""
from dataclasses import dataclass, asdict
import math


@dataclass(frozen=True)
class ChannelConfig:
    nnx: int            # streamwise points (nnx/2 complex modes kept)
    nny: int            # spanwise points (nny complex modes, Nyquist unused)
    nnz: int            # Chebyshev degree; nnz+1 wall-normal points
    aphi: float         # streamwise box = 2*pi*aphi   (paraandcons.f90:22)
    beta: float         # spanwise box   = 2*pi*beta   (paraandcons.f90:22)
    dt: float           # time step                    (paraandcons.f90:23)
    re: float           # Reynolds number, viscosity 1/re (paraandcons.f90:24)
    re_p: float         # constant mean pressure gradient (paraandcons.f90:25)

    def __post_init__(self):
        if self.nnx % 4 or self.nny % 4 or self.nnx < 4 or self.nny < 4:
            raise ValueError("nnx and nny must be positive multiples of 4")
        if self.nnz < 4:
            raise ValueError("nnz must be >= 4")
        for n in (3 * self.nnx // 2, 3 * self.nny // 2, 4 * self.nnz):
            m = n
            for p in (2, 3, 5):
                while m % p == 0:
                    m //= p
            if m != 1:
                raise ValueError(f"transform length {n} must factor into 2, 3 and 5")

    @property
    def kx(self) -> int:
        return self.nnx // 2

    @property
    def points(self) -> int:
        """Grid points per step: nnx * nny * (nnz+1)."""
        return self.nnx * self.nny * (self.nnz + 1)

    def as_dict(self):
        return asdict(self)


def _laminar_rep(re_c: float) -> float:
    # U = 1 - z^2 is steady when re_p = -(1/re) U'' = 2/re.
    return 2.0 / re_c


# The benchmark configurations, with their reference-parameter equivalents.
CONFIGS = {
    # 32 x 33 x 32, box 2pi x 2 x pi, Re_c = 2000, dt = 1e-3.
    "c1_poiseuille_32": ChannelConfig(32, 32, 32, 1.0, 0.5, 1e-3, 2000.0, _laminar_rep(2000.0)),
    # 16 x 65 x 4, box 2pi x 2 x 2pi, Re_c = 7500, dt = 1e-3.
    "c2_orr_sommerfeld": ChannelConfig(16, 4, 64, 1.0, 1.0, 1e-3, 7500.0, _laminar_rep(7500.0)),
    # 128 x 129 x 128, box 4pi x 2 x 4pi/3, Re_tau = 180 (re = 180, re_p = 1).  dt = 2e-4 as in
    # the reference's own run (paraandcons.f90:23): at dt = 5e-4 the reference algorithm
    # diverges within ~45 steps from a 10% perturbation at this resolution (the highest
    # streamwise, spanwise and Chebyshev modes grow about tenfold per step).
    "c3_retau180_128": ChannelConfig(128, 128, 128, 2.0, 2.0 / 3.0, 2e-4, 180.0, 1.0),
    # 384 x 193 x 384, box 2pi x 2 x pi, Re_tau = 550.  dt = 5e-5: from the
    # wall-law mean with 10% fluctuations the reference algorithm (AB2
    # nonlinear term) diverges at dt = 2e-4 within 40 steps and at 1e-4 within
    # about 120; at 5e-5 the energy stays within 0.3% over 200 steps.
    "c4_retau550_384": ChannelConfig(384, 384, 192, 1.0, 0.5, 5e-5, 550.0, 1.0),
}


def small(nnx=16, nny=8, nnz=16, aphi=1.0, beta=0.5, dt=1e-3, re=180.0, re_p=1.0) -> ChannelConfig:
    return ChannelConfig(nnx, nny, nnz, aphi, beta, dt, re, re_p)


def grid_points_per_step(cfg: ChannelConfig) -> int:
    return cfg.points


def pi() -> float:
    return math.pi
