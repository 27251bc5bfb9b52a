"""Float64 restatement of somax's multilayer shallow-water right-hand side (test infrastructure).

This module is the checker of the GPU shallow-water kernels, not product code.  It follows
``somax/_src/models/swm/multilayer.py``:

* ``vector_field``               :150-200 (mass, PV, cross-velocity PV fluxes, Bernoulli
                                  potential with the cumulative hydrostatic pressure, wind on the
                                  top layer over H[0], harmonic diffusion, bottom drag)
* ``apply_boundary_conditions``  :202-219 and the wall helpers :366-410
* ``diagnose``                   :221-257
* ``create``                     :259-363 (grid, f(y) and the wind pattern at T rows)

The operators are finitevolx v0.0.39's (``Advection2D`` upwind1, ``Vorticity2D``,
``Interpolation2D``, ``Difference2D``, ``Diffusion2D``, ``kinetic_energy``), which the
reference does not vendor.  They are restated on the Arakawa C-grid that
``ArakawaCGrid2D.from_interior`` describes: T points at cell centres (j, i), U points on east
faces (j, i + 1/2), V points on north faces (j + 1/2, i), X points on north-east corners
(j + 1/2, i + 1/2), arrays (..., Ny, Nx) with one ghost ring.  Every operator writes the
interior [1:-1, 1:-1] and leaves the ring zero (finitevolx's interior-write convention, the
same one the QG restatement uses for its Laplacian); the face fluxes of the upwind advection
are formed on every face an interior cell needs.  Parity with the reference for these
stencils is unpinned (no live finitevolx); the reference's own tests of this model (rest
state, wind on the top layer only, pressure coupling between layers, wall rules, finite
integration, non-negative energy) are restated in ``tests/test_oracle_swm.py``.
"""

from __future__ import annotations

import dataclasses

import numpy as np

from . import qg as _qg

S = (Ellipsis, slice(1, -1), slice(1, -1))


def _interior(shape_like: np.ndarray, inner: np.ndarray) -> np.ndarray:
    out = np.zeros_like(shape_like)
    out[S] = inner
    return out


# ---- Interpolation2D (interior write) -------------------------------------------------
def T_to_U(a):
    return _interior(a, 0.5 * (a[..., 1:-1, 1:-1] + a[..., 1:-1, 2:]))


def T_to_V(a):
    return _interior(a, 0.5 * (a[..., 1:-1, 1:-1] + a[..., 2:, 1:-1]))


def T_to_X(a):
    return _interior(a, 0.25 * (a[..., 1:-1, 1:-1] + a[..., 1:-1, 2:] + a[..., 2:, 1:-1] + a[..., 2:, 2:]))


def X_to_U(a):
    return _interior(a, 0.5 * (a[..., 1:-1, 1:-1] + a[..., :-2, 1:-1]))


def X_to_V(a):
    return _interior(a, 0.5 * (a[..., 1:-1, 1:-1] + a[..., 1:-1, :-2]))


def V_to_U(a):
    return _interior(a, 0.25 * (a[..., 1:-1, 1:-1] + a[..., 1:-1, 2:] + a[..., :-2, 1:-1] + a[..., :-2, 2:]))


def U_to_V(a):
    return _interior(a, 0.25 * (a[..., 1:-1, 1:-1] + a[..., 1:-1, :-2] + a[..., 2:, 1:-1] + a[..., 2:, :-2]))


def U_to_T(a):
    return _interior(a, 0.5 * (a[..., 1:-1, 1:-1] + a[..., 1:-1, :-2]))


def V_to_T(a):
    return _interior(a, 0.5 * (a[..., 1:-1, 1:-1] + a[..., :-2, 1:-1]))


# ---- Difference2D / Vorticity2D / kinetic_energy / Diffusion2D / Advection2D ------------
def diff_x_T_to_U(a, dx):
    return _interior(a, (a[..., 1:-1, 2:] - a[..., 1:-1, 1:-1]) / dx)


def diff_y_T_to_V(a, dy):
    return _interior(a, (a[..., 2:, 1:-1] - a[..., 1:-1, 1:-1]) / dy)


def relative_vorticity(u, v, dx, dy):
    """zeta at X points: d_x v - d_y u."""
    return _interior(u, (v[..., 1:-1, 2:] - v[..., 1:-1, 1:-1]) / dx - (u[..., 2:, 1:-1] - u[..., 1:-1, 1:-1]) / dy)


def potential_vorticity(u, v, h, f, dx, dy):
    """q = (zeta + f) / h at X points, f and h interpolated from T points."""
    zeta = relative_vorticity(u, v, dx, dy)
    hX, fX = T_to_X(h), T_to_X(f)
    out = np.zeros_like(u)
    out[S] = (zeta[S] + fX[S]) / hX[S]
    return out


def kinetic_energy(u, v):
    """KE at T points: (U_to_T(u^2) + V_to_T(v^2)) / 2."""
    return 0.5 * (U_to_T(u * u) + V_to_T(v * v))


def diffusion(a, nu, dx, dy):
    """nu lap(a), 5-point, interior."""
    return nu * _qg.laplacian(a, dx, dy)


def advection_upwind1(h, u, v, dx, dy):
    """-div(h u, h v) with first-order upwind h on every face (the mass equation)."""
    hx = np.where(u[..., :, :-1] > 0, h[..., :, :-1], h[..., :, 1:])  # face i + 1/2, i = 0 .. Nx - 2
    hy = np.where(v[..., :-1, :] > 0, h[..., :-1, :], h[..., 1:, :])  # face j + 1/2
    F = u[..., :, :-1] * hx
    G = v[..., :-1, :] * hy
    inner = -((F[..., 1:-1, 1:] - F[..., 1:-1, :-1]) / dx + (G[..., 1:, 1:-1] - G[..., :-1, 1:-1]) / dy)
    return _interior(h, inner)


# ---- model ---------------------------------------------------------------------------
@dataclasses.dataclass
class SWModel:
    nx: int
    ny: int
    Lx: float
    Ly: float
    f0: float
    beta: float
    H: np.ndarray
    g_prime: np.ndarray
    lateral_viscosity: float
    bottom_drag: float
    wind_amplitude: float
    wind_profile: str = "doublegyre"
    bc: str = "periodic"

    @property
    def Nx(self):
        return self.nx + 2

    @property
    def Ny(self):
        return self.ny + 2

    @property
    def dx(self):
        return self.Lx / self.nx

    @property
    def dy(self):
        return self.Ly / self.ny

    @property
    def nl(self):
        return len(self.H)

    def y(self):
        return np.arange(self.Ny) * self.dy

    def f_field(self):
        """f at T points, f0 + beta (y - Ly / 2) (``coriolis_fn``, multilayer.py:331-335)."""
        return np.broadcast_to((self.f0 + self.beta * (self.y() - self.Ly / 2.0))[:, None], (self.Ny, self.Nx))

    def wind_stress_x(self):
        """-cos(2 pi y / Ly) (double gyre) or -cos(pi y / Ly) (single), multilayer.py:338-342."""
        k = 2.0 if self.wind_profile != "single" else 1.0
        return np.broadcast_to((-np.cos(k * np.pi * self.y() / self.Ly))[:, None], (self.Ny, self.Nx))


def create(nx=64, ny=64, Lx=4e6, Ly=4e6, f0=9.375e-5, beta=1.754e-11, H=(400.0, 1100.0, 2600.0),
           g_prime=(9.81, 0.025, 0.0125), lateral_viscosity=0.0, bottom_drag=0.0, wind_amplitude=0.0,
           wind_profile="doublegyre", bc="periodic") -> SWModel:
    """``MultilayerShallowWater2D.create`` defaults (multilayer.py:259-278)."""
    if len(H) != len(g_prime):
        raise ValueError("H and g_prime must have the same length")
    return SWModel(nx, ny, Lx, Ly, f0, beta, np.asarray(H, float), np.asarray(g_prime, float), lateral_viscosity,
                   bottom_drag, wind_amplitude, wind_profile, bc)


def _periodic(a):
    a = a.copy()
    a[..., 0, :] = a[..., -2, :]
    a[..., -1, :] = a[..., 1, :]
    a[..., :, 0] = a[..., :, -2]
    a[..., :, -1] = a[..., :, 1]
    return a


def apply_boundary_conditions(m: SWModel, h, u, v):
    """Periodic wrap of every field, or the wall rules (multilayer.py:381-404): u = 0 on the
    west ring, the east wall face and the east ring, then free slip in y; v = 0 on the south
    ring, the north wall face and the north ring, then free slip in x; h zero-gradient."""
    if m.bc == "periodic":
        return _periodic(h), _periodic(u), _periodic(v)
    u = u.copy()
    v = v.copy()
    h = h.copy()
    u[..., :, 0] = 0.0
    u[..., :, -2] = 0.0
    u[..., :, -1] = 0.0
    u[..., 0, :] = u[..., 1, :]
    u[..., -1, :] = u[..., -2, :]
    v[..., 0, :] = 0.0
    v[..., -2, :] = 0.0
    v[..., -1, :] = 0.0
    v[..., :, 0] = v[..., :, 1]
    v[..., :, -1] = v[..., :, -2]
    h[..., 0, :] = h[..., 1, :]
    h[..., -1, :] = h[..., -2, :]
    h[..., :, 0] = h[..., :, 1]
    h[..., :, -1] = h[..., :, -2]
    return h, u, v


def vector_field(m: SWModel, h, u, v, params: dict | None = None):
    """(dh, du, dv) of ``MultilayerShallowWater2D.vector_field`` (multilayer.py:150-200) on the
    state as given (no BC here; ``_rhs`` applies it first)."""
    p = params or {}
    nu = p.get("lateral_viscosity", m.lateral_viscosity)
    kappa = p.get("bottom_drag", m.bottom_drag)
    tau0 = p.get("wind_amplitude", m.wind_amplitude)
    dx, dy = m.dx, m.dy
    t = h.dtype  # float64 by default; float32 gives the FP32 floor of a comparison
    dh = advection_upwind1(h, u, v, dx, dy)
    f = np.broadcast_to(m.f_field().astype(t), h.shape)
    q = potential_vorticity(u, v, h, f, dx, dy)
    uh = T_to_U(h) * u
    vh = T_to_V(h) * v
    qU, qV = X_to_U(q), X_to_V(q)
    vhU, uhV = V_to_U(vh), U_to_V(uh)
    ke = kinetic_energy(u, v)
    pres = np.cumsum(m.g_prime.astype(t)[:, None, None] * h, axis=0)
    P = ke + pres
    du = qU * vhU - diff_x_T_to_U(P, dx)
    dv = -qV * uhV - diff_y_T_to_V(P, dy)
    du[0] += (tau0 * m.wind_stress_x() / m.H[0]).astype(t)
    # wind_stress_y is zero (multilayer.py:343)
    du = du + diffusion(u, t.type(nu), dx, dy)
    dv = dv + diffusion(v, t.type(nu), dx, dy)
    du[-1] -= t.type(kappa) * u[-1]
    dv[-1] -= t.type(kappa) * v[-1]
    return dh, du, dv


def rhs(m: SWModel, y: np.ndarray, params: dict | None = None) -> np.ndarray:
    """``_rhs`` on a stacked state y = (3, nl, Ny, Nx) = (h, u, v): BC, then the tendencies."""
    h, u, v = apply_boundary_conditions(m, y[0], y[1], y[2])
    return np.stack(vector_field(m, h, u, v, params))


def integrate(m: SWModel, y0: np.ndarray, dt: float, n_steps: int, scheme: str = "tsit5",
              params: dict | None = None) -> np.ndarray:
    """``SomaxModel.integrate`` with a constant step on the stacked state: BC on the initial
    state, BC on every stage input, the final state as stepped."""
    h, u, v = apply_boundary_conditions(m, y0[0], y0[1], y0[2])
    y = np.stack([h, u, v])
    for _ in range(n_steps):
        y = _qg.rk_step(lambda z: rhs(m, z, params), y, dt, scheme)
    return y


def diagnose(m: SWModel, h, u, v) -> dict:
    """Energy (KE + g' h^2 / 2) and potential enstrophy (q^2 h_X / 2) per layer
    (multilayer.py:221-257)."""
    area = m.dx * m.dy
    ke = kinetic_energy(u, v)
    zeta = relative_vorticity(u, v, m.dx, m.dy)
    f = np.broadcast_to(m.f_field(), h.shape)
    q = potential_vorticity(u, v, h, f, m.dx, m.dy)
    hX = T_to_X(h)
    ke_sum = np.sum(ke[S], axis=(-2, -1)) * area
    pe_sum = 0.5 * m.g_prime * np.sum(h[S] ** 2, axis=(-2, -1)) * area
    energy = ke_sum + pe_sum
    ens = 0.5 * np.sum(q[S] ** 2 * hX[S], axis=(-2, -1)) * area
    return dict(energy=energy, total_energy=energy.sum(), enstrophy=ens, total_enstrophy=ens.sum(),
                potential_vorticity=q, relative_vorticity=zeta, kinetic_energy_field=ke)


# ---- float64 derivatives (the checker of the hand-written shallow-water adjoint) -------------
SWM_PARAMS = ("lateral_viscosity", "bottom_drag", "wind_amplitude")


def _rhs_flat(m: SWModel, y: np.ndarray, params: dict | None, apply_bc: bool) -> np.ndarray:
    if apply_bc:
        return rhs(m, y, params).reshape(-1)
    return np.stack(vector_field(m, y[0], y[1], y[2], params)).reshape(-1)


def rhs_jacobian(m: SWModel, y: np.ndarray, params: dict | None = None, apply_bc: bool = True,
                 rel: float = 1e-6) -> np.ndarray:
    """Dense Jacobian of ``rhs`` (apply_bc: the boundary rules applied to y first) by central
    differences with a step of ``rel`` times each field's largest magnitude.  The right-hand side
    is smooth away from the upwind switch (u = 0 on a face), which the tests' states avoid; the
    differences are then exact to O(step^2)."""
    y = np.asarray(y, dtype=np.float64)
    n = y.size
    scale = [max(np.abs(y[f]).max(), 1e-3) * rel for f in range(3)]
    per_field = n // 3
    J = np.empty((n, n))
    flat = y.reshape(-1)
    for c in range(n):
        h = scale[c // per_field]
        yp = flat.copy()
        ym = flat.copy()
        yp[c] += h
        ym[c] -= h
        J[:, c] = (_rhs_flat(m, yp.reshape(y.shape), params, apply_bc) -
                   _rhs_flat(m, ym.reshape(y.shape), params, apply_bc)) / (2.0 * h)
    return J


def rhs_param_derivatives(m: SWModel, y: np.ndarray, apply_bc: bool = True) -> np.ndarray:
    """d rhs / d (nu, kappa, tau0), (3, n): the right-hand side is affine in each parameter, so
    a forward difference of a unit step is exact up to rounding."""
    base = {k: float(getattr(m, k)) for k in SWM_PARAMS}
    f0 = _rhs_flat(m, y, base, apply_bc)
    out = []
    for k in SWM_PARAMS:
        p = dict(base)
        p[k] += 1.0
        out.append(_rhs_flat(m, y, p, apply_bc) - f0)
    return np.stack(out)


def step_jacobian(m: SWModel, y: np.ndarray, dt: float, n_steps: int, scheme: str, rel: float = 1e-6) -> np.ndarray:
    """Dense Jacobian of n_steps constant steps (no initial boundary rules: a step continues an
    integration) by central differences, as ``rhs_jacobian``."""
    y = np.asarray(y, dtype=np.float64)
    n = y.size
    scale = [max(np.abs(y[f]).max(), 1e-3) * rel for f in range(3)]
    per_field = n // 3
    flat = y.reshape(-1)

    def run(z):
        z = z.reshape(y.shape)
        for _ in range(n_steps):
            z = _qg.rk_step(lambda w: rhs(m, w), z, dt, scheme)
        return z.reshape(-1)

    J = np.empty((n, n))
    for c in range(n):
        h = scale[c // per_field]
        yp = flat.copy()
        ym = flat.copy()
        yp[c] += h
        ym[c] -= h
        J[:, c] = (run(yp) - run(ym)) / (2.0 * h)
    return J
