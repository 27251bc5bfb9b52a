"""Float64 restatement of the geostrophic projection of ``ReparameterizedQG``
(``somax/_src/models/qg/reparameterized.py:142-178``): test infrastructure (the oracle).

P = G (Q G)^-1 Q on a multilayer shallow-water state (h, u, v), arrays (nl, Ny, Nx) with the
ghost ring, as the reference computes it:

* Q (``reparameterized.py:160-166``): q = zeta - f0 (h - H) / H, zeta the relative vorticity
  ``Vorticity2D.relative_vorticity(u, v)`` (finitevolx v0.0.39, not vendored) at the C-grid
  corner points, dv/dx - du/dy with u on the east faces and v on the north faces of T-cell
  (j, i) and the corner (j, i) north-east of it: zeta[j, i] = (v[j, i+1] - v[j, i]) / dx -
  (u[j+1, i] - u[j, i]) / dy on interior cells, zero on the ring;
* (Q G)^-1 (``reparameterized.py:125-140``): the modal Helmholtz inversion of
  ``BaroclinicQG._invert_pv`` (``oracle.qg.invert_pv``: to_modal, DST-I with lambda_m =
  f0^2 eig_m, to_layer, zero ring);
* G (``reparameterized.py:169-176``): (u_g, v_g) = ``Difference2D.grad_perp(psi)`` =
  (-d psi/dy at the u points, d psi/dx at the v points) = (-(psi[j, i] - psi[j-1, i]) / dy,
  (psi[j, i] - psi[j, i-1]) / dx) on interior cells, zero on the ring, and
  h_g = H (1 + f0 Cm2l diag(eig) Cl2m psi).

The stencils of zeta and grad_perp are the published C-grid operators; parity with finitevolx
is unpinned beyond the reference's tests (rest state a fixed point, projection idempotent to
discretisation error, finite, non-zero geostrophic velocity for a height anomaly,
``tests/models/test_qg_reparameterized.py:61-117``), which the tests restate.  With these
stencils curl(grad_perp psi) is exactly the 5-point Laplacian of psi on the interior.
"""

from __future__ import annotations

import numpy as np

from oracle import qg as O


def relative_vorticity(u: np.ndarray, v: np.ndarray, dx: float, dy: float) -> np.ndarray:
    """zeta = dv/dx - du/dy at the corner points, interior cells; zero ring."""
    z = np.zeros(np.broadcast_shapes(u.shape, v.shape), dtype=np.result_type(u, v))
    z[..., 1:-1, 1:-1] = (v[..., 1:-1, 2:] - v[..., 1:-1, 1:-1]) / dx - (u[..., 2:, 1:-1] - u[..., 1:-1, 1:-1]) / dy
    return z


def grad_perp(psi: np.ndarray, dx: float, dy: float) -> tuple[np.ndarray, np.ndarray]:
    """(u, v) = (-d psi/dy at the u points, d psi/dx at the v points), interior; zero ring."""
    u = np.zeros_like(psi)
    v = np.zeros_like(psi)
    u[..., 1:-1, 1:-1] = -(psi[..., 1:-1, 1:-1] - psi[..., :-2, 1:-1]) / dy
    v[..., 1:-1, 1:-1] = (psi[..., 1:-1, 1:-1] - psi[..., 1:-1, :-2]) / dx
    return u, v


def pv_of(m: O.QGModel, h: np.ndarray, u: np.ndarray, v: np.ndarray) -> np.ndarray:
    """Q: q = zeta - f0 (h - H) / H (``reparameterized.py:160-166``)."""
    g = m.grid
    H = np.asarray(m.H, dtype=np.float64)[:, None, None]
    return relative_vorticity(u, v, g.dx, g.dy) - m.f0 * (h - H) / H


def project(m: O.QGModel, h: np.ndarray, u: np.ndarray, v: np.ndarray):
    """``ReparameterizedQG.project``: returns (h_g, u_g, v_g, psi)."""
    if m.barotropic:
        raise ValueError("the projection is defined for the multilayer (baroclinic) model")
    g = m.grid
    psi = O.invert_pv(m, pv_of(m, h, u, v))
    ug, vg = grad_perp(psi, g.dx, g.dy)
    H = np.asarray(m.H, dtype=np.float64)[:, None, None]
    ev = m.modes.eigenvalues[:, None, None]
    a_psi = m.modes.to_layer(ev * m.modes.to_modal(psi))
    hg = H * (1.0 + m.f0 * a_psi)
    return hg, ug, vg, psi


def integrate(m: O.QGModel, ms, y0: np.ndarray, dt: float, n_steps: int, scheme: str = "tsit5") -> np.ndarray:
    """``ReparameterizedQG`` through ``SomaxModel.integrate`` with constant steps on the stacked
    state y = (3, nl, Ny, Nx) = (h, u, v): ``apply_boundary_conditions`` (the SWM wall rules,
    then the projection; ``reparameterized.py:186-189``) on the initial state and on every stage
    input before the shallow-water ``vector_field`` (``reparameterized.py:180-184``); ``m`` is
    the QG model of the projection's inversion, ``ms`` the ``oracle.swm`` model (wall BC)."""
    from oracle import swm as W

    def bc(y):
        h, u, v = W.apply_boundary_conditions(ms, y[0], y[1], y[2])
        return np.stack(project(m, h, u, v)[:3])

    y = bc(np.asarray(y0, dtype=np.float64))
    for _ in range(n_steps):
        y = O.rk_step(lambda z: np.stack(W.vector_field(ms, *bc(z))), y, dt, scheme)
    return y
