"""Workload definitions and the initial-state generator.

The reference hard-codes its parameters in ``srcs/main.f90:91-249`` and builds
its initial state with ``init`` (``srcs/init.f:1-45``), ``init_phi``
(``srcs/init_phi_legendre.f90:1-31``) and ``init_array_x_stripe``
(``srcs/init_array_x_stripe.f90:1-60``).  This module replaces those with a
seeded, host-side generator whose arrays are handed unchanged to both the
CUDA library and the CPU oracle, so the two start from identical bits.

Axis convention (reference order): ``i`` = x (periodic), ``j`` = wall-normal
(walls at j=0|1 and j=nj|nj+1), ``k`` = the second periodic direction.  The
workloads below are stated in that order; a workload quoted as
``nx x ny x nz`` with walls in z maps to ``(ni, nj, nk) = (nx, nz, ny)`` and
domain ``(xl, yl, zl) = (Lx, Lz, Ly)``.

Every 3-D array is Fortran-ordered with origin -2: numpy shape
``(nk+6, nj+6, ni+6)`` in C order, element ``(i, j, k)`` at
``a[k+2, j+2, i+2]``.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

STATE_FIELDS = ("u", "v", "w", "uo", "vo", "wo", "p", "po", "phi0", "phi1", "phin0", "phin1")


@dataclasses.dataclass
class Config:
    name: str
    ni: int
    nj: int
    nk: int
    xl: float
    yl: float
    zl: float
    dt: float
    steps: int
    rhol: float = 1.0       # fluid at phi=0
    rhog: float = 1.0       # fluid at phi=1 (the pressure Poisson uses this one)
    rmul: float = 0.05
    rmug: float = 0.05
    sigma: float = 1.0
    uwall: float = -1.0     # lower wall moves at -uwall, upper at +uwall (bndu.f:47,81)
    slip: float = 0.1       # slip length l1 = l2
    zeta_coef: float | None = 0.1  # GNBC friction coefficient zeta (None: main.f90:172 formula)
    theta_lo: float = 90.0  # static angle, lower wall (deg)
    theta_hi: float = 90.0  # static angle, upper wall (deg)
    init: str = "stripe"    # stripe | stripe_perturbed | droplet
    seed: int = 0
    bet_mthinc: float = 2.0
    checker_cells: int = 0  # >0: lower-wall 60/120 deg checkerboard of this many cells
    theta_noise_deg: float = 0.0
    grvb: float = 0.0
    grvp: float = 0.0
    harmonic: int = 0

    @property
    def dx(self) -> float:
        return self.xl / self.ni

    @property
    def dy(self) -> float:
        return self.yl / self.nj

    @property
    def dz(self) -> float:
        return self.zl / self.nk

    @property
    def shape(self) -> tuple:
        return (self.nk + 6, self.nj + 6, self.ni + 6)

    @property
    def cells(self) -> int:
        return self.ni * self.nj * self.nk

    @property
    def zeta(self) -> float:
        """Contact-line friction coefficient of the GNBC law cos(theta_d) = cos(theta_0) -
        zeta*u_cl/sigma (gnbc.f90:47).  The workloads state one "GNBC slip coefficient" of
        0.1; it is used both as this zeta and as the Navier slip length (bndu.f:39-45).
        zeta_coef=None falls back to the reference's own formula (main.f90:172)."""
        if self.zeta_coef is not None:
            return self.zeta_coef
        return 0.21 * 6.0 * (self.rmul / self.slip + self.rmug / self.slip)

    def scaled(self, ni: int, nj: int, nk: int, **kw) -> "Config":
        return dataclasses.replace(self, ni=ni, nj=nj, nk=nk, **kw)


def _check_pow2(n: int) -> None:
    # main.f90:117-126: every grid dimension must be a power of two
    if n < 4 or n & (n - 1):
        raise ValueError(f"grid size {n} must be a power of two >= 4")


# The five workloads (reference axis order).
WORKLOADS = {
    # two-phase Couette, x-stripe, equal properties, CPU-runnable: 32x16x32, walls in z
    "couette32": Config("couette32", 32, 32, 16, 2.0, 1.0, 1.0, dt=1e-4, steps=100),
    # 256x128x128, density and viscosity ratio 10, perturbed stripe, 60 deg
    "couette256": Config("couette256", 256, 128, 128, 2.0, 1.0, 1.0, dt=2e-5, steps=1000,
                         rhol=10.0, rhog=1.0, rmul=0.5, rmug=0.05, theta_lo=60.0, theta_hi=60.0,
                         init="stripe_perturbed", seed=1234),
    # 512x256x256 sessile droplet on a 60/120 deg checkerboard lower wall (0.125 squares)
    "droplet512": Config("droplet512", 512, 256, 256, 2.0, 1.0, 1.0, dt=1e-5, steps=500,
                         rhol=1000.0, rhog=1.0, rmul=0.5, rmug=0.005, uwall=0.0,
                         theta_lo=60.0, theta_hi=90.0, init="droplet", checker_cells=32),
    # 128x64x64 Couette geometry of couette32, per-wall-cell angle 75 + N(0, 5^2) deg
    "couette128": Config("couette128", 128, 64, 64, 2.0, 1.0, 1.0, dt=1e-4, steps=200,
                         theta_lo=75.0, theta_hi=75.0, theta_noise_deg=5.0, seed=77),
    # the droplet scaled to 256x128x128
    "droplet256": Config("droplet256", 256, 128, 128, 2.0, 1.0, 1.0, dt=1e-5, steps=500,
                         rhol=1000.0, rhog=1.0, rmul=0.5, rmug=0.005, uwall=0.0,
                         theta_lo=60.0, theta_hi=90.0, init="droplet", checker_cells=16),
}


def get(name: str, **overrides) -> Config:
    cfg = WORKLOADS[name]
    return dataclasses.replace(cfg, **overrides) if overrides else cfg


def empty(cfg: Config, n: int = 1) -> np.ndarray:
    shape = cfg.shape if n == 1 else (n,) + cfg.shape
    return np.zeros(shape, dtype=np.float64)


def interior(a: np.ndarray) -> np.ndarray:
    return a[..., 3:-3, 3:-3, 3:-3]


def phi_interior(cfg: Config) -> np.ndarray:
    """Initial volume fraction (phi=1: the rhog fluid) on the interior cells, shape (nk,nj,ni)."""
    x = (np.arange(1, cfg.ni + 1) - 0.5) * cfg.dx
    y = (np.arange(1, cfg.nj + 1) - 0.5) * cfg.dy
    z = (np.arange(1, cfg.nk + 1) - 0.5) * cfg.dz
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    width = 1.5 * cfg.dx
    if cfg.init in ("stripe", "stripe_perturbed"):
        shift = np.zeros_like(X)
        if cfg.init == "stripe_perturbed":
            rng = np.random.default_rng(cfg.seed)
            for m in range(5):
                for n in range(5):
                    if m == 0 and n == 0:
                        continue
                    a = rng.normal(0.0, 0.01)
                    ph = rng.uniform(0.0, 2.0 * math.pi)
                    # modes along the periodic direction (z_ref, period zl) and the
                    # wall-normal direction (y_ref, period yl)
                    shift += a * np.cos(2.0 * math.pi * (m * Z / cfg.zl + n * Y / cfg.yl) + ph)
        d = 0.5 * cfg.xl / 2.0 - np.abs(X - 0.5 * cfg.xl - shift)
        return 0.5 * (1.0 + np.tanh(d / width))
    if cfg.init == "droplet":
        # spherical cap of radius 0.3 centred at x=xl/2, z=zl/2, 0.15 above the lower wall;
        # the drop is the rhol fluid (phi=0), the surroundings phi=1.
        r = np.sqrt((X - 0.5 * cfg.xl) ** 2 + (Y - 0.15) ** 2 + (Z - 0.5 * cfg.zl) ** 2)
        inside = 0.5 * (1.0 + np.tanh((0.3 - r) / width))
        return 1.0 - inside
    raise ValueError(cfg.init)


def wall_arrays(cfg: Config):
    """theta0, zeta, l1, l2 as full halo'd 3-D arrays (only the j=1 and j=nj planes are read).

    Mirrors init_array_x_stripe.f90:21-47 in where the values live: lower wall at j=1,
    upper wall at j=nj, every i and k of those planes including halos.
    """
    th = empty(cfg)
    ze = empty(cfg)
    l1 = empty(cfg)
    l2 = empty(cfg)
    jl, jh = 1 + 2, cfg.nj + 2
    th[:, jl, :] = cfg.theta_lo
    th[:, jh, :] = cfg.theta_hi
    if cfg.checker_cells > 0:
        ii = np.arange(-2, cfg.ni + 4)
        kk = np.arange(-2, cfg.nk + 4)
        pi_ = ((ii + cfg.ni - 1) // cfg.checker_cells)[None, :]
        pk_ = ((kk + cfg.nk - 1) // cfg.checker_cells)[:, None]
        th[:, jl, :] = np.where((pi_ + pk_) % 2 == 0, 60.0, 120.0)
    if cfg.theta_noise_deg > 0.0:
        rng = np.random.default_rng(cfg.seed + 1)
        noise = rng.normal(0.0, cfg.theta_noise_deg, size=(2, cfg.nk + 6, cfg.ni + 6))
        th[:, jl, :] += noise[0]
        th[:, jh, :] += noise[1]
    for a in (ze,):
        a[:, jl, :] = cfg.zeta
        a[:, jh, :] = cfg.zeta
    for a in (l1, l2):
        a[:, jl, :] = cfg.slip
        a[:, jh, :] = cfg.slip
    return th, ze, l1, l2


def raw_state(cfg: Config) -> np.ndarray:
    """State stack (12, nk+6, nj+6, ni+6) before the start-up boundary pass.

    u=v=w=p=uo=vo=wo=po=0 (init.f:18-42); phi1 from phi_interior with periodic
    x/z halos; phi0 and phin* zero (phin is never initialised before the first
    step in the reference, main.f90:303-370, and its allocation is zero-filled).
    """
    for n in (cfg.ni, cfg.nj, cfg.nk):
        _check_pow2(n)
    st = np.zeros((12,) + cfg.shape, dtype=np.float64)
    phi1 = st[STATE_FIELDS.index("phi1")]
    phi1[3:-3, 3:-3, 3:-3] = phi_interior(cfg)
    periodic(phi1, cfg)
    return st


def periodic(q: np.ndarray, cfg: Config) -> None:
    """bnd_periodic.f:166-208 on a numpy array (x halos, then z halos)."""
    ni, nk = cfg.ni, cfg.nk
    # x: q(-2..0) = q(ni-2..ni), q(ni+1..ni+3) = q(1..3)
    q[:, :, 0:3] = q[:, :, ni - 2 + 2:ni + 1 + 2]
    q[:, :, ni + 3:ni + 6] = q[:, :, 3:6]
    q[0:3, :, :] = q[nk - 2 + 2:nk + 1 + 2, :, :]
    q[nk + 3:nk + 6, :, :] = q[3:6, :, :]
