"""NumPy/SciPy restatement of somax's multilayer QG hot path (the oracle).

Test infrastructure only.  Every function names the reference code it follows.  Arrays use
the reference layout: ``(..., Ny, Nx)`` with axis -2 = y, axis -1 = x, ``Ny = ny + 2`` and
``Nx = nx + 2`` (one ghost ring), ``dx = Lx / nx`` and ``dy = Ly / ny``.

All functions are dtype-generic: float64 inputs give the FP64 oracle, float32 inputs give the
FP32 CPU path that stands in for the reference's default (JAX without x64) when timed.

Conventions that the reference fixes by printed outputs (parity pinned):
  * DST-I Helmholtz over the FULL array, ring included (tutorial step10 cells 4/12,
    step11 cell 6).
  * 5-point Laplacian on the interior + classical RK stepping (tutorial step07: energy
    decay and the gradient dL/dnu).
Conventions that no reference test pins (parity unpinned, published methods used):
  * Arakawa (1966) Jacobian normalisation/axis order, ring output of the Laplacian (zero),
    the coupling matrix A, C-grid diagnostics.
"""

from __future__ import annotations

import dataclasses
import math
from typing import Callable, Sequence

import numpy as np
import scipy.fft as sfft

# ----------------------------------------------------------------------------------------
# Grid and boundary helpers
# ----------------------------------------------------------------------------------------


@dataclasses.dataclass(frozen=True)
class Grid:
    """Arakawa C-grid with one ghost ring (finitevolx ``ArakawaCGrid2D.from_interior``).

    ``from_interior(nx, ny, Lx, Ly)`` gives ``Nx = nx + 2``, ``dx = Lx / nx``; the tutorial
    print-out ``ArakawaCGrid2D(Nx=66, Ny=66, Lx=4.0, Ly=4.0, dx=0.0625, dy=0.0625)``
    (``content/tutorials/step07_diffusion_2d.ipynb`` cell 5) pins this.
    """

    nx: int
    ny: int
    Lx: float
    Ly: float

    @property
    def Nx(self) -> int:
        return self.nx + 2

    @property
    def Ny(self) -> int:
        return self.ny + 2

    @property
    def dx(self) -> float:
        return self.Lx / self.nx

    @property
    def dy(self) -> float:
        return self.Ly / self.ny


def zero_boundaries(a: np.ndarray) -> np.ndarray:
    """Zero the ghost ring (finitevolx ``zero_boundaries``; pinned by
    ``tests/models/test_qg_baroclinic.py:166-183``)."""
    out = np.array(a, copy=True)
    out[..., 0, :] = 0
    out[..., -1, :] = 0
    out[..., :, 0] = 0
    out[..., :, -1] = 0
    return out


def enforce_periodic(a: np.ndarray) -> np.ndarray:
    """Periodic ghost ring (finitevolx ``enforce_periodic``, used by
    ``somax/_src/models/pde2d/diffusion.py:67-69``): ghosts copy the opposite interior edge."""
    out = np.array(a, copy=True)
    out[..., 0, :] = out[..., -2, :]
    out[..., -1, :] = out[..., 1, :]
    out[..., :, 0] = out[..., :, -2]
    out[..., :, -1] = out[..., :, 1]
    return out


# ----------------------------------------------------------------------------------------
# Finite-difference operators
# ----------------------------------------------------------------------------------------


def laplacian(a: np.ndarray, dx: float, dy: float) -> np.ndarray:
    """5-point Laplacian on the interior, zero on the ghost ring.

    finitevolx ``Difference2D.laplacian`` as called at ``baroclinic.py:184,188`` and
    ``barotropic.py:146,150``.  The interior formula is pinned by the step07 diffusion
    tutorial; the zero ring output is the finitevolx interior-write convention (unpinned).
    """
    a = np.asarray(a)
    out = np.zeros_like(a)
    c = a[..., 1:-1, 1:-1]
    out[..., 1:-1, 1:-1] = (a[..., 1:-1, 2:] - 2 * c + a[..., 1:-1, :-2]) / dx**2 + (
        a[..., 2:, 1:-1] - 2 * c + a[..., :-2, 1:-1]
    ) / dy**2
    return out


def arakawa_jacobian(f: np.ndarray, g: np.ndarray, dx: float, dy: float) -> np.ndarray:
    """Arakawa (1966) energy- and enstrophy-conserving Jacobian J(f, g) = f_x g_y - f_y g_x.

    Called as ``arakawa_jacobian(psi, q + beta*y, dx, dy)`` at ``baroclinic.py:174-175`` and
    ``barotropic.py:136-137``; returns the interior ``(..., Ny-2, Nx-2)`` which the caller
    scatters into zeros (``baroclinic.py:176-178``).  The sign J = f_x g_y - f_y g_x follows
    from u = -psi_y, v = psi_x (``barotropic.py:88-91``).  The average of the three
    second-order forms J++, J+x, Jx+ is the published scheme.
    """
    f = np.asarray(f)
    g = np.asarray(g)

    def s(a, dj, di):
        ny, nx = a.shape[-2], a.shape[-1]
        return a[..., 1 + dj : ny - 1 + dj, 1 + di : nx - 1 + di]

    # (dj, di) offsets: j along y (axis -2), i along x (axis -1)
    fE, fW, fN, fS = s(f, 0, 1), s(f, 0, -1), s(f, 1, 0), s(f, -1, 0)
    gE, gW, gN, gS = s(g, 0, 1), s(g, 0, -1), s(g, 1, 0), s(g, -1, 0)
    fNE, fNW, fSE, fSW = s(f, 1, 1), s(f, 1, -1), s(f, -1, 1), s(f, -1, -1)
    gNE, gNW, gSE, gSW = s(g, 1, 1), s(g, 1, -1), s(g, -1, 1), s(g, -1, -1)

    jpp = (fE - fW) * (gN - gS) - (fN - fS) * (gE - gW)
    jpx = fE * (gNE - gSE) - fW * (gNW - gSW) - fN * (gNE - gNW) + fS * (gSE - gSW)
    jxp = gN * (fNE - fNW) - gS * (fSE - fSW) - gE * (fNE - fSE) + gW * (fNW - fSW)
    return (jpp + jpx + jxp) / (12.0 * dx * dy)


# ----------------------------------------------------------------------------------------
# DST-I Helmholtz inversion (finitevolx pv_inversion / streamfunction_from_vorticity)
# ----------------------------------------------------------------------------------------


def dst1_eigenvalues(n: int, d: float) -> np.ndarray:
    """Eigenvalues of the 1-D 3-point second difference with Dirichlet zeros at -1 and n:
    (2 cos(pi k / (n + 1)) - 2) / d^2, k = 1..n."""
    k = np.arange(1, n + 1, dtype=np.float64)
    return (2.0 * np.cos(np.pi * k / (n + 1)) - 2.0) / d**2


def dst1_matrix(n: int) -> np.ndarray:
    """Orthonormal DST-I matrix S[i, j] = sqrt(2/(n+1)) sin(pi (i+1)(j+1)/(n+1)); S @ S = I."""
    k = np.arange(1, n + 1, dtype=np.float64)
    return math.sqrt(2.0 / (n + 1)) * np.sin(np.pi * np.outer(k, k) / (n + 1))


def helmholtz_dst(rhs: np.ndarray, dx: float, dy: float, lam: float | np.ndarray = 0.0) -> np.ndarray:
    """Solve (nabla^2 - lam) phi = rhs by DST-I over the FULL (Ny, Nx) array.

    Restates finitevolx ``streamfunction_from_vorticity(..., bc="dst", lambda_=lam)``
    (``barotropic.py:119-121``, ``pde2d/poisson.py:38,131-133``) and ``pv_inversion``
    (``baroclinic.py:146-152``).  The full-array convention (ghost ring included, Dirichlet
    zeros implied at indices -1 and N) reproduces the tutorial outputs to 6-7 digits.
    ``lam`` may be an array broadcasting against the leading axes (one value per mode).
    """
    rhs = np.asarray(rhs)
    dt = rhs.dtype if np.issubdtype(rhs.dtype, np.floating) else np.float64
    ny, nx = rhs.shape[-2], rhs.shape[-1]
    ex = dst1_eigenvalues(nx, dx).astype(dt)
    ey = dst1_eigenvalues(ny, dy).astype(dt)
    lam = np.asarray(lam, dtype=dt)
    if lam.ndim:
        lam = lam.reshape(lam.shape + (1, 1))
    hat = sfft.dstn(rhs, type=1, axes=(-2, -1), workers=_WORKERS)
    hat = hat / (ey[:, None] + ex[None, :] - lam)
    return sfft.idstn(hat, type=1, axes=(-2, -1), workers=_WORKERS).astype(dt, copy=False)


def helmholtz_apply_full(phi: np.ndarray, dx: float, dy: float, lam: float | np.ndarray = 0.0) -> np.ndarray:
    """The operator that ``helmholtz_dst`` inverts: full-array 5-point Laplacian with zeros
    outside the array, minus lam * phi.  Used for residuals."""
    phi = np.asarray(phi)
    p = np.pad(phi, [(0, 0)] * (phi.ndim - 2) + [(1, 1), (1, 1)])
    c = p[..., 1:-1, 1:-1]
    lap = (p[..., 1:-1, 2:] - 2 * c + p[..., 1:-1, :-2]) / dx**2 + (p[..., 2:, 1:-1] - 2 * c + p[..., :-2, 1:-1]) / dy**2
    lam = np.asarray(lam, dtype=phi.dtype)
    if lam.ndim:
        lam = lam.reshape(lam.shape + (1, 1))
    return lap - lam * phi


_WORKERS = 1


def set_workers(n: int) -> None:
    """Thread count for scipy.fft inside the oracle (CPU baseline timing)."""
    global _WORKERS
    _WORKERS = int(n)


# ----------------------------------------------------------------------------------------
# Vertical modes (somax/_src/core/transforms.py + finitevolx build_coupling_matrix /
# decompose_vertical_modes)
# ----------------------------------------------------------------------------------------


def coupling_matrix(H: Sequence[float], g_prime: Sequence[float]) -> np.ndarray:
    """Layer coupling matrix A of the stretching term (finitevolx ``build_coupling_matrix``,
    called at ``transforms.py:192``).  Textbook tridiagonal form of the layered QG
    stretching operator (MQGeometry), top interface g'[0]: (A psi)_k couples layer k to
    k-1 through g'[k] and to k+1 through g'[k+1]."""
    H = np.asarray(H, dtype=np.float64)
    g = np.asarray(g_prime, dtype=np.float64)
    n = H.size
    A = np.zeros((n, n))
    if n == 1:
        A[0, 0] = 1.0 / (H[0] * g[0])
        return A
    A[0, 0] = 1.0 / (H[0] * g[0]) + 1.0 / (H[0] * g[1])
    A[0, 1] = -1.0 / (H[0] * g[1])
    for k in range(1, n - 1):
        A[k, k - 1] = -1.0 / (H[k] * g[k])
        A[k, k] = (1.0 / g[k] + 1.0 / g[k + 1]) / H[k]
        A[k, k + 1] = -1.0 / (H[k] * g[k + 1])
    A[n - 1, n - 2] = -1.0 / (H[n - 1] * g[n - 1])
    A[n - 1, n - 1] = 1.0 / (H[n - 1] * g[n - 1])
    return A


@dataclasses.dataclass
class Modes:
    """``ModalTransform`` (``transforms.py:151-224``): Cl2m, Cm2l, eigenvalues, radii."""

    Cl2m: np.ndarray
    Cm2l: np.ndarray
    eigenvalues: np.ndarray
    rossby_radii: np.ndarray

    def to_modal(self, x: np.ndarray) -> np.ndarray:  # transforms.py:218-220
        return np.einsum("lm,m...->l...", self.Cl2m.astype(x.dtype), x)

    def to_layer(self, x: np.ndarray) -> np.ndarray:  # transforms.py:222-224
        return np.einsum("lm,m...->l...", self.Cm2l.astype(x.dtype), x)


def vertical_modes(H, g_prime, f0: float, eigs: str = "consistent") -> Modes:
    """``ModalTransform.from_physics`` (``transforms.py:172-200``).

    Cm2l holds the right eigenvectors of A (sorted by ascending eigenvalue), Cl2m = Cm2l^-1
    (so Cl2m @ Cm2l = I, ``test_transforms.py:133-137``).  The column scaling of Cm2l does
    not change the inversion (it cancels in Cm2l diag(.) Cl2m).

    ``eigs="consistent"``: Helmholtz eigenvalues = eig(A), paired with the modes.
    ``eigs="reference"``: the reference takes them from ``jnp.linalg.eigh(A)``
    (``transforms.py:194``), which symmetrises A; reproduced as eigvalsh((A + A^T)/2).
    """
    A = coupling_matrix(H, g_prime)
    lam, R = np.linalg.eig(A)
    lam = lam.real
    R = R.real
    order = np.argsort(lam)
    lam = lam[order]
    R = R[:, order]
    Cm2l = R
    Cl2m = np.linalg.inv(R)
    with np.errstate(divide="ignore", invalid="ignore"):
        radii = 1.0 / (f0 * np.sqrt(lam))
    if eigs == "consistent":
        ev = lam
    elif eigs == "reference":
        ev = np.linalg.eigvalsh(0.5 * (A + A.T))
    else:
        raise ValueError(f"unknown eigs mode {eigs!r}")
    return Modes(Cl2m=Cl2m, Cm2l=Cm2l, eigenvalues=ev, rossby_radii=radii)


def modes_from_N2_constant(N2: float, depth: float, n_layers: int, g: float = 9.81):
    """``StratificationProfile.from_N2_constant`` (``transforms.py:41-76``): equal layers,
    g'[0] = g, g'[k>=1] = N2 * H_k."""
    Hk = depth / n_layers
    H = np.full(n_layers, Hk)
    gp = np.concatenate([[g], np.full(n_layers - 1, N2 * Hk)])
    return H, gp


# ----------------------------------------------------------------------------------------
# Models
# ----------------------------------------------------------------------------------------


@dataclasses.dataclass
class QGModel:
    """Everything ``BaroclinicQG.create`` / ``BarotropicQG.create`` precompute
    (``baroclinic.py:230-332``, ``barotropic.py:186-248``) plus two extensions: biharmonic
    viscosity ``nu4`` (-nu4 lap(lap q)) and an optional land mask (1 = ocean)."""

    grid: Grid
    f0: float
    beta: float
    H: np.ndarray
    g_prime: np.ndarray
    modes: Modes | None  # None: barotropic (pure Poisson, ring of psi kept)
    lateral_viscosity: float = 0.0
    bottom_drag: float = 0.0
    wind_amplitude: float = 0.0
    biharmonic_viscosity: float = 0.0
    wind_profile: str = "doublegyre"

    @property
    def barotropic(self) -> bool:
        return self.modes is None

    @property
    def nl(self) -> int:
        return 1 if self.modes is None else self.modes.Cl2m.shape[0]

    @property
    def helmholtz_lambdas(self) -> np.ndarray:
        """f0^2 * eigenvalues (``baroclinic.py:296``); zero for the barotropic model."""
        if self.modes is None:
            return np.zeros(1)
        return self.f0**2 * self.modes.eigenvalues

    def beta_y(self, dtype=np.float64) -> np.ndarray:
        """beta (y - Ly/2) with y = j dy (``baroclinic.py:307-311``)."""
        g = self.grid
        y = np.arange(g.Ny, dtype=np.float64) * g.dy
        Y = np.broadcast_to(y[:, None], (g.Ny, g.Nx))
        return (self.beta * (Y - g.Ly / 2.0)).astype(dtype)

    def wind_forcing(self, dtype=np.float64) -> np.ndarray:
        """Normalised wind-stress curl (``baroclinic.py:313-318``)."""
        g = self.grid
        y = np.arange(g.Ny, dtype=np.float64) * g.dy
        Y = np.broadcast_to(y[:, None], (g.Ny, g.Nx))
        if self.wind_profile == "single":
            F = np.sin(np.pi * Y / g.Ly)
        else:
            F = -np.sin(2.0 * np.pi * Y / g.Ly)
        return F.astype(dtype)


def baroclinic_model(
    nx=64, ny=64, Lx=4e6, Ly=4e6, f0=9.375e-5, beta=1.754e-11,
    H=(400.0, 1100.0, 2600.0), g_prime=(9.81, 0.025, 0.0125),
    lateral_viscosity=0.0, bottom_drag=0.0, wind_amplitude=0.0,
    biharmonic_viscosity=0.0, wind_profile="doublegyre", eigs="consistent",
) -> QGModel:
    """``BaroclinicQG.create`` defaults (``baroclinic.py:231-247``)."""
    if len(H) != len(g_prime):
        raise ValueError("H and g_prime must have the same length")
    modes = vertical_modes(H, g_prime, f0, eigs=eigs)
    return QGModel(Grid(nx, ny, Lx, Ly), f0, beta, np.asarray(H, float), np.asarray(g_prime, float), modes,
                   lateral_viscosity, bottom_drag, wind_amplitude, biharmonic_viscosity, wind_profile)


def barotropic_model(
    nx=64, ny=64, Lx=1e6, Ly=1e6, f0=1e-4, beta=1.6e-11,
    lateral_viscosity=0.0, bottom_drag=0.0, wind_amplitude=0.0,
    biharmonic_viscosity=0.0, wind_profile="doublegyre",
) -> QGModel:
    """``BarotropicQG.create`` defaults (``barotropic.py:186-197``)."""
    return QGModel(Grid(nx, ny, Lx, Ly), f0, beta, np.ones(1), np.ones(1), None,
                   lateral_viscosity, bottom_drag, wind_amplitude, biharmonic_viscosity, wind_profile)


def invert_pv(m: QGModel, q: np.ndarray) -> np.ndarray:
    """``BaroclinicQG._invert_pv`` (``baroclinic.py:135-159``): to_modal, per-mode DST-I
    Helmholtz with lambda_m = f0^2 eig_m, to_layer, zero ring.
    Barotropic (``barotropic.py:113-121``): Poisson, ring kept."""
    g = m.grid
    if m.barotropic:
        return helmholtz_dst(q, g.dx, g.dy, 0.0)
    qm = m.modes.to_modal(q)
    pm = helmholtz_dst(qm, g.dx, g.dy, m.helmholtz_lambdas.astype(q.dtype))
    psi = m.modes.to_layer(pm)
    return zero_boundaries(psi)


def vector_field(m: QGModel, q: np.ndarray, params: dict | None = None) -> np.ndarray:
    """dq/dt (``baroclinic.py:161-190``, ``barotropic.py:123-152``).  No BC is applied to
    ``q`` here, exactly like the reference's ``vector_field``.  ``params`` may override the
    differentiable parameters (``lateral_viscosity``, ``bottom_drag``, ``wind_amplitude``)
    and the extension ``biharmonic_viscosity``."""
    p = dict(lateral_viscosity=m.lateral_viscosity, bottom_drag=m.bottom_drag,
             wind_amplitude=m.wind_amplitude, biharmonic_viscosity=m.biharmonic_viscosity)
    if params:
        p.update(params)
    dt = q.dtype
    g = m.grid
    nu, kappa, tau0, nu4 = (dt.type(p[k]) for k in ("lateral_viscosity", "bottom_drag", "wind_amplitude", "biharmonic_viscosity"))
    psi = invert_pv(m, q)
    by = m.beta_y(dt)
    F = m.wind_forcing(dt)
    if m.barotropic:
        J = arakawa_jacobian(psi, q + by, g.dx, g.dy)
        dq = np.zeros_like(q)
        dq[1:-1, 1:-1] = J
        dq = -dq
        dq = dq + tau0 * F
        dq = dq - kappa * laplacian(psi, g.dx, g.dy)
        lq = laplacian(q, g.dx, g.dy)
        dq = dq + nu * lq
        if nu4 != 0:
            dq = dq - nu4 * laplacian(lq, g.dx, g.dy)
        return dq
    J = arakawa_jacobian(psi, q + by[None], g.dx, g.dy)
    dq = np.zeros_like(q)
    dq[:, 1:-1, 1:-1] = J
    dq = -dq
    dq[0] = dq[0] + tau0 * F / dt.type(m.H[0])
    dq[-1] = dq[-1] + (-kappa) * laplacian(psi[-1], g.dx, g.dy)
    lq = laplacian(q, g.dx, g.dy)
    dq = dq + nu * lq
    if nu4 != 0:
        dq = dq - nu4 * laplacian(lq, g.dx, g.dy)
    return dq


def apply_boundary_conditions(m: QGModel, q: np.ndarray) -> np.ndarray:
    """``baroclinic.py:192-195`` / ``barotropic.py:154-157``: zero ring."""
    return zero_boundaries(q)


# ----------------------------------------------------------------------------------------
# Time stepping (core/model.py:39-88: BC on every stage input; diffrax schemes)
# ----------------------------------------------------------------------------------------

# Tsitouras (2011) 5(4) tableau as used by diffrax.Tsit5 (published coefficients).
_TSIT5_C = [0.0, 0.161, 0.327, 0.9, 0.9800255409045097, 1.0, 1.0]
_TSIT5_A = [
    [],
    [0.161],
    [-0.008480655492356989, 0.335480655492357],
    [2.897153057105493, -6.359448489975075, 4.3622954328695815],
    [5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525],
    [5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383],
    [0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081, 2.324710524099774],
]
_TSIT5_B = [0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081, 2.324710524099774, 0.0]

SCHEMES = ("euler", "heun", "ssprk3", "tsit5")


def rk_step(f: Callable[[np.ndarray], np.ndarray], y0: np.ndarray, dt: float, scheme: str) -> np.ndarray:
    """One explicit RK step of y' = f(y).  ``f`` must already apply the BC to its input
    (``core/model.py:47-49``).

    heun   : diffrax ``Heun`` (c = [0, 1], b = [1/2, 1/2]).
    ssprk3 : Shu-Osher SSP-RK3 (historical ``mqg_demo_retangular.ipynb`` cell 31).
    tsit5  : diffrax ``Tsit5`` (default solver, ``core/model.py:75``), constant steps.
    """
    t = y0.dtype.type
    dt = t(dt)
    if scheme == "euler":
        return y0 + dt * f(y0)
    if scheme == "heun":
        k1 = f(y0)
        k2 = f(y0 + dt * k1)
        return y0 + dt * (t(0.5) * k1 + t(0.5) * k2)
    if scheme == "ssprk3":
        y1 = y0 + dt * f(y0)
        y2 = t(0.75) * y0 + t(0.25) * (y1 + dt * f(y1))
        return t(1.0 / 3.0) * y0 + t(2.0 / 3.0) * (y2 + dt * f(y2))
    if scheme == "tsit5":
        ks = []
        for s in range(7):
            if s == 0:
                ys = y0
            else:
                acc = np.zeros_like(y0)
                for j, a in enumerate(_TSIT5_A[s]):
                    acc = acc + t(a) * ks[j]
                ys = y0 + dt * acc
            if s == 6:
                break  # b_7 = 0: the 7th stage only feeds FSAL
            ks.append(f(ys))
        acc = np.zeros_like(y0)
        for j in range(6):
            acc = acc + t(_TSIT5_B[j]) * ks[j]
        return y0 + dt * acc
    raise ValueError(f"unknown scheme {scheme!r}")


def integrate(m: QGModel, q0: np.ndarray, dt: float, n_steps: int, scheme: str = "ssprk3",
              params: dict | None = None, save_every: int | None = None):
    """``SomaxModel.integrate`` (``core/model.py:53-88``) with ``ConstantStepSize``:
    BC on the initial state, BC on every RHS input, final state returned as stepped (its
    ring is not re-zeroed).  Returns the final state, or a stack of states saved every
    ``save_every`` steps."""

    def f(y):
        return vector_field(m, apply_boundary_conditions(m, y), params)

    y = apply_boundary_conditions(m, q0)
    saved = []
    for i in range(n_steps):
        y = rk_step(f, y, dt, scheme)
        if save_every and (i + 1) % save_every == 0:
            saved.append(y.copy())
    return np.stack(saved) if save_every else y


# ----------------------------------------------------------------------------------------
# Diagnostics (baroclinic.py:197-228, barotropic.py:159-183)
# ----------------------------------------------------------------------------------------


def diagnose(m: QGModel, q: np.ndarray) -> dict:
    """KE and enstrophy per layer.  u = -d_y psi on V points, v = d_x psi on U points
    (finitevolx ``diff_y_T_to_V`` / ``diff_x_T_to_U``, forward differences written to the
    interior), averaged back to T points (``V_to_T`` / ``U_to_T``: mean of the two faces);
    KE = 1/2 sum_interior (u_T^2 + v_T^2) dx dy, enstrophy = 1/2 sum_interior q^2 dx dy.
    The C-grid staggering is the finitevolx convention (unpinned)."""
    g = m.grid
    psi = invert_pv(m, q)
    u = np.zeros_like(psi)
    v = np.zeros_like(psi)
    u[..., 1:-1, 1:-1] = -(psi[..., 2:, 1:-1] - psi[..., 1:-1, 1:-1]) / g.dy
    v[..., 1:-1, 1:-1] = (psi[..., 1:-1, 2:] - psi[..., 1:-1, 1:-1]) / g.dx
    uT = np.zeros_like(u)
    vT = np.zeros_like(v)
    uT[..., 1:-1, 1:-1] = 0.5 * (u[..., 1:-1, 1:-1] + u[..., :-2, 1:-1])
    vT[..., 1:-1, 1:-1] = 0.5 * (v[..., 1:-1, 1:-1] + v[..., 1:-1, :-2])
    area = g.dx * g.dy
    s = (Ellipsis, slice(1, -1), slice(1, -1))
    ke = 0.5 * np.sum(uT[s] ** 2 + vT[s] ** 2, axis=(-2, -1)) * area
    ens = 0.5 * np.sum(q[s] ** 2, axis=(-2, -1)) * area
    return dict(psi=psi, u=u, v=v, kinetic_energy=ke, enstrophy=ens,
                total_kinetic_energy=np.sum(ke), total_enstrophy=np.sum(ens),
                relative_vorticity=laplacian(psi, g.dx, g.dy))


def integrate_and_compare(case: dict) -> float:
    """Process-pool worker of the ensemble parity tests: integrates one member in float64 and
    returns the interior relative L2 distance of ``case["got"]`` from it.  ``case`` holds the
    keyword arguments of ``baroclinic_model`` (``model``), the initial PV (``q0``), ``dt``,
    ``n_steps``, ``scheme`` and the state to check (``got``)."""
    set_workers(case.get("workers", 1))
    m = baroclinic_model(**case["model"])
    ref = integrate(m, np.asarray(case["q0"], np.float64), case["dt"], case["n_steps"], case["scheme"])
    got = np.asarray(case["got"], np.float64)
    s = (Ellipsis, slice(1, -1), slice(1, -1))
    return float(np.linalg.norm(got[s] - ref[s]) / np.linalg.norm(ref[s]))
