"""Seeded synthetic workloads of the QG time step (double-gyre basins) and of the multilayer
shallow-water model.

Shapes and parameters of the QG benchmark configurations; the initial PV is a seeded
Gaussian random field with an isotropic k^-3 spectrum (no dataset is involved).  Wind
amplitudes follow the reference factory's convention: ``wind_amplitude = tau0 * 2 pi /
(rho0 * Ly)`` with the ``-sin(2 pi y / Ly)`` double-gyre pattern
(``somax/_src/models/gfd_testcases.py:250-251``, ``baroclinic.py:316-318``).
"""

from __future__ import annotations

import dataclasses
import math

import numpy as np
import scipy.fft as sfft

RHO0 = 1000.0
L_BASIN = 5.12e6
F0 = 9.375e-5
BETA = 1.754e-11


def wind_amplitude(tau0: float, Ly: float = L_BASIN, rho0: float = RHO0) -> float:
    """Wind-stress curl amplitude of a tau0 (N/m^2) double gyre."""
    return tau0 * 2.0 * math.pi / (rho0 * Ly)


@dataclasses.dataclass
class QGConfig:
    name: str
    n: int                       # interior cells per side
    H: tuple
    g_prime: tuple
    dt: float
    scheme: str
    lateral_viscosity: float = 0.0
    biharmonic_viscosity: float = 0.0
    bottom_drag: float = 1e-7
    tau0: float = 0.08
    L: float = L_BASIN

    @property
    def nl(self) -> int:
        return len(self.H)

    @property
    def steps_per_day(self) -> float:
        return 86400.0 / self.dt

    def model_kwargs(self) -> dict:
        return dict(nx=self.n, ny=self.n, Lx=self.L, Ly=self.L, f0=F0, beta=BETA, n_layers=self.nl,
                    H=tuple(self.H), g_prime=tuple(self.g_prime), lateral_viscosity=self.lateral_viscosity,
                    bottom_drag=self.bottom_drag, wind_amplitude=wind_amplitude(self.tau0, self.L),
                    biharmonic_viscosity=self.biharmonic_viscosity)


# Barotropic double gyre with a 50 km deformation radius: a 1-layer model with
# g' = (f0 Rd)^2 / H so that f0^2 / (g' H) = 1 / Rd^2.
RD_C1 = 5.0e4
C1 = QGConfig("barotropic_64", 64, (4000.0,), ((F0 * RD_C1) ** 2 / 4000.0,), 4000.0, "heun",
              lateral_viscosity=100.0)
C2 = QGConfig("baroclinic3_128", 128, (400.0, 1100.0, 2600.0), (9.81, 0.025, 0.0125), 1200.0, "ssprk3",
              biharmonic_viscosity=2e9)
C3_512 = dataclasses.replace(C2, name="baroclinic3_512", n=512)
C3_1024 = dataclasses.replace(C2, name="baroclinic3_1024", n=1024)
C5 = dataclasses.replace(C2, name="baroclinic3_256", n=256)
# Five layers, H geometric from 200 m to 2000 m; reduced gravities chosen to decrease with
# depth (the configuration leaves them open).
H5 = tuple(float(200.0 * 10 ** (k / 4)) for k in range(5))
G5 = (9.81, 0.030, 0.020, 0.0125, 0.008)
C4_MIX = (
    (96, dataclasses.replace(C1, name="ens_barotropic_64", dt=1200.0, scheme="ssprk3")),
    (96, dataclasses.replace(C2, name="ens_baroclinic3_128")),
    (48, dataclasses.replace(C2, name="ens_baroclinic3_256", n=256)),
    (16, dataclasses.replace(C2, name="ens_baroclinic5_256", n=256, H=H5, g_prime=G5)),
)
CONFIGS = {c.name: c for c in (C1, C2, C3_512, C3_1024, C5)}


def c4_members(seed: int = 0) -> list:
    """The 256 members of the configuration-4 ensemble in order: (config, tau0 in N/m^2,
    PV seed) per member, tau0 drawn uniformly from 0.05-0.12 N/m^2 with a seeded generator.
    Member k's initial PV is ``initial_pv(config, pv_seed)``."""
    rng = np.random.default_rng(1000 + seed)
    out = []
    for count, cfg in C4_MIX:
        for _ in range(count):
            out.append((cfg, float(rng.uniform(0.05, 0.12)), 10000 * seed + len(out)))
    return out


def member_kwargs(cfg: QGConfig, tau0: float | None = None) -> dict:
    """``model_kwargs`` of a configuration with the wind amplitude of ``tau0`` (N/m^2)."""
    kw = cfg.model_kwargs()
    if tau0 is not None:
        kw["wind_amplitude"] = wind_amplitude(tau0, cfg.L)
    return kw


def kminus3_field(n: int, seed: int, nl: int = 1) -> np.ndarray:
    """(nl, n+2, n+2) float64 fields, zero ring, unit RMS interior, with power spectrum
    proportional to k^-3 over the interior DST-I wavenumbers."""
    rng = np.random.default_rng(seed)
    k = np.arange(1, n + 1, dtype=np.float64)
    kk = np.sqrt(k[:, None] ** 2 + k[None, :] ** 2)
    amp = kk ** -1.5
    out = np.zeros((nl, n + 2, n + 2))
    for l in range(nl):
        c = rng.standard_normal((n, n)) * amp
        f = sfft.idstn(c, type=1, norm="ortho")
        out[l, 1:-1, 1:-1] = f / np.sqrt(np.mean(f * f))
    return out


def initial_pv(cfg: QGConfig, seed: int = 0, rms_vorticity: float = 1e-6) -> np.ndarray:
    """Seeded k^-3 PV with RMS relative vorticity ``rms_vorticity`` in the top layer.

    The relative vorticity of a PV field q is lap(psi) with (lap - lambda) psi = q; its RMS
    is evaluated spectrally on the interior (Dirichlet) modes with the barotropic-mode
    lambda.  Deeper layers are scaled by H[0] / H[k] (thicker layers carry weaker PV
    anomalies).
    """
    n = cfg.n
    f = kminus3_field(n, seed, cfg.nl)
    d = cfg.L / n
    k = np.arange(1, n + 1)
    e = (2 * np.cos(np.pi * k / (n + 1)) - 2) / d**2
    E = e[:, None] + e[None, :]
    if cfg.nl == 1:
        lam = F0**2 / (cfg.g_prime[0] * cfg.H[0])
    else:
        lam = 0.0
    c = sfft.dstn(f[0, 1:-1, 1:-1], type=1, norm="ortho")
    zeta = sfft.idstn(c * E / (E - lam), type=1, norm="ortho")
    scale = rms_vorticity / np.sqrt(np.mean(zeta**2))
    for l in range(cfg.nl):
        f[l] *= scale * cfg.H[0] / cfg.H[l]
    return f


def land_mask(ny: int, nx: int, frac: float = 0.15, seed: int = 0, n_blobs: int = 8) -> np.ndarray:
    """(ny + 2, nx + 2) uint8 land mask of a masked basin (1 = ocean): the ring is land and
    ``n_blobs`` connected land blobs grown from seeded centres cover ``frac`` of the interior
    T-cells.  A blob is the set of cells within r(theta) = R (1 + 0.15 sin(3 theta + a) +
    0.1 sin(5 theta + b)) of its centre (a wavy coastline); all blobs grow together (R scaled
    by bisection) until the land fraction is reached."""
    rng = np.random.default_rng(seed)
    Ny, Nx = ny + 2, nx + 2
    cy = rng.uniform(0.1, 0.9, n_blobs) * ny + 1
    cx = rng.uniform(0.1, 0.9, n_blobs) * nx + 1
    rel = rng.uniform(0.6, 1.4, n_blobs)
    ph = rng.uniform(0, 2 * math.pi, (n_blobs, 2))
    jj, ii = np.mgrid[0:Ny, 0:Nx]
    dist = []
    for b in range(n_blobs):
        dy, dx = jj - cy[b], ii - cx[b]
        th = np.arctan2(dy, dx)
        shape = rel[b] * (1 + 0.15 * np.sin(3 * th + ph[b, 0]) + 0.1 * np.sin(5 * th + ph[b, 1]))
        dist.append(np.hypot(dy, dx) / shape)
    dmin = np.min(dist, axis=0)[1:-1, 1:-1]
    target = frac * ny * nx
    lo, hi = 0.0, float(max(ny, nx))
    for _ in range(60):
        mid = 0.5 * (lo + hi)
        if (dmin <= mid).sum() < target:
            lo = mid
        else:
            hi = mid
    mask = np.ones((Ny, Nx), np.uint8)
    mask[1:-1, 1:-1][dmin <= hi] = 0
    mask[0, :] = mask[-1, :] = mask[:, 0] = mask[:, -1] = 0
    return mask


# ---- multilayer shallow-water workloads ----------------------------------------------------
@dataclasses.dataclass
class SWMConfig:
    """A shallow-water basin stepped with constant steps; one bench step = ``bench_steps``."""

    name: str
    n: int
    L: float
    H: tuple
    g_prime: tuple
    f0: float
    beta: float
    lateral_viscosity: float
    bottom_drag: float
    wind_amplitude: float
    bc: str
    dt: float
    scheme: str
    bench_steps: int
    initial: str  # "jet" (baroclinic_instability_swm) or "bump" (rest + seeded height anomaly)

    @property
    def nl(self) -> int:
        return len(self.H)

    def model_kwargs(self) -> dict:
        return dict(nx=self.n, ny=self.n, Lx=self.L, Ly=self.L, f0=self.f0, beta=self.beta, n_layers=self.nl,
                    H=tuple(self.H), g_prime=tuple(self.g_prime), lateral_viscosity=self.lateral_viscosity,
                    bottom_drag=self.bottom_drag, wind_amplitude=self.wind_amplitude, bc=self.bc)

    def oracle_kwargs(self) -> dict:
        kw = self.model_kwargs()
        kw.pop("n_layers")
        return kw


# The 2-layer baroclinic jet of the reference's run configuration ``swm_jet`` (64^2 periodic
# basin of 1000 km, nu = 1000 m^2/s, dt = 20 s, 30 days saved daily; the runner integrates with
# the default Tsit5): one bench step = one model day = 4320 steps.
SWM_JET64 = SWMConfig("swm_jet64", 64, 1.0e6, (500.0, 4500.0), (9.81, 0.025), 1e-4, 1.6e-11, 1000.0, 1e-7, 0.0,
                      "periodic", 20.0, "tsit5", 4320, "jet")
# A 3-layer 1024^2 wall-bounded double gyre of 4000 km (the reparameterised double gyre's
# stratification and wind, 3.9 km cells) from rest with a seeded height anomaly; dt = 10 s
# (0.5 of the external gravity-wave CFL), one bench step = one model hour = 360 steps.
SWM3_1024 = SWMConfig("swm3_1024", 1024, 4.0e6, (400.0, 1100.0, 2600.0), (9.81, 0.025, 0.0125), F0, BETA, 100.0,
                      3.6e-8, 8e-5, "wall", 10.0, "tsit5", 360, "bump")
SWM_CONFIGS = {c.name: c for c in (SWM_JET64, SWM3_1024)}


def swm_initial_state(cfg: SWMConfig, seed: int = 0) -> np.ndarray:
    """(3, nl, n+2, n+2) float32 (h, u, v): the jet of ``baroclinic_instability_swm`` or the
    rest state plus a k^-3 height anomaly of 2 m peak per layer."""
    N = cfg.n + 2
    dx = cfg.L / cfg.n
    if cfg.initial == "jet":
        x = np.arange(N) * dx
        env = np.exp(-0.5 * ((np.arange(N) * dx - cfg.L / 2.0) / 5e4) ** 2)[:, None] * np.ones((1, N))
        u = np.stack([s * 0.5 * env for s in (1.0, -1.0)])
        v = np.stack([0.01 * np.sin(4.0 * math.pi * x / cfg.L)[None, :] * env] * 2)
        h = np.asarray(cfg.H, float)[:, None, None] * np.ones((cfg.nl, N, N))
        return np.stack([h, u, v]).astype(np.float32)
    k = kminus3_field(cfg.n, seed, cfg.nl)
    h = np.asarray(cfg.H, float)[:, None, None] + 2.0 * k / np.abs(k).max()
    z = np.zeros_like(h)
    return np.stack([h, z, z]).astype(np.float32)
