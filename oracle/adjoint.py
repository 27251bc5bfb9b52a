"""Float64 derivatives of the oracle, the checker of the hand-written adjoints (test
infrastructure only).

The reference takes these derivatives with JAX autodiff (``eqx.filter_grad`` through
``integrate``: ``tests/models/test_qg_baroclinic.py:293-312``).  JAX is not available here,
so the oracle gets them from its own float64 forward:

* the RHS is quadratic in q (J(psi, q) with psi linear in q) and affine in each parameter,
  so central differences of ``qg.vector_field`` are exact up to float64 rounding: the dense
  Jacobian column j is ``(F(q + h e_j) - F(q - h e_j)) / 2h`` for any h, and the parameter
  derivative is ``(F(p + h e_k) - F(p)) / h`` for any h;
* the inversion is linear: its matrix column j is ``invert(e_j)``;
* through many steps the map is not polynomial; there the oracle gives central differences
  with a small relative step, whose truncation error is O(h^2).  The same float64
  central-difference construction reproduces the gradient the reference's tutorial prints
  with autodiff (``content/tutorials/step07_diffusion_2d.ipynb`` cell 18) to 1e-6.
"""

from __future__ import annotations

import numpy as np

from . import qg as O

PARAM_NAMES = ("lateral_viscosity", "bottom_drag", "wind_amplitude", "biharmonic_viscosity")


def _params(m: O.QGModel, params: dict | None) -> dict:
    p = {k: float(getattr(m, k)) for k in PARAM_NAMES}
    if params:
        p.update(params)
    return p


def rhs(m: O.QGModel, q: np.ndarray, params: dict | None = None, apply_bc: bool = False) -> np.ndarray:
    """``vector_field`` (apply_bc: of the ring-zeroed q, ``core/model.py:47-49``)."""
    if apply_bc:
        q = O.apply_boundary_conditions(m, q)
    return O.vector_field(m, q, _params(m, params))


def rhs_jacobian(m: O.QGModel, q: np.ndarray, params: dict | None = None, apply_bc: bool = False) -> np.ndarray:
    """Dense d rhs / d q (n x n, n = q.size) by exact central differences."""
    q = np.asarray(q, np.float64)
    n = q.size
    h = max(float(np.abs(q).max()), 1e-30)
    Jm = np.empty((n, n))
    e = np.zeros(n)
    for j in range(n):
        e[j] = h
        Jm[:, j] = ((rhs(m, q + e.reshape(q.shape), params, apply_bc) -
                     rhs(m, q - e.reshape(q.shape), params, apply_bc)) / (2 * h)).reshape(-1)
        e[j] = 0.0
    return Jm


def rhs_param_derivatives(m: O.QGModel, q: np.ndarray, params: dict | None = None,
                          apply_bc: bool = False, scale: float = 1.0) -> np.ndarray:
    """d rhs / d p_k for the four parameters (4 x n).  rhs is affine in each parameter, so a
    difference over any step is exact; the step is sized so the change is 1e3 x |rhs|
    (rounding relative to the derivative stays ~1e-13)."""
    q = np.asarray(q, np.float64)
    p = _params(m, params)
    base = rhs(m, q, p, apply_bc)
    fn = max(float(np.linalg.norm(base)), 1e-300)
    out = []
    for k in PARAM_NAMES:
        pk = dict(p)
        pk[k] = p[k] + 1.0
        g1 = rhs(m, q, pk, apply_bc) - base
        h = scale * 1e3 * fn / max(float(np.linalg.norm(g1)), 1e-300)
        pk[k] = p[k] + h
        out.append(((rhs(m, q, pk, apply_bc) - base) / h).reshape(-1))
    return np.stack(out)


def rhs_vjp(m: O.QGModel, q: np.ndarray, g: np.ndarray, params: dict | None = None, apply_bc: bool = False):
    """(q_bar, params_bar) of ``rhs`` for the cotangent g (dense; small grids only)."""
    Jm = rhs_jacobian(m, q, params, apply_bc)
    G = rhs_param_derivatives(m, q, params, apply_bc)
    gv = np.asarray(g, np.float64).reshape(-1)
    return (Jm.T @ gv).reshape(np.shape(q)), G @ gv


def rhs_directional(m: O.QGModel, q: np.ndarray, d: np.ndarray, params: dict | None = None,
                    apply_bc: bool = False) -> np.ndarray:
    """(d rhs / d q) d, exact for the quadratic rhs (any grid size)."""
    q = np.asarray(q, np.float64)
    d = np.asarray(d, np.float64)
    h = max(float(np.abs(q).max()), 1e-30) / max(float(np.abs(d).max()), 1e-300)
    return (rhs(m, q + h * d, params, apply_bc) - rhs(m, q - h * d, params, apply_bc)) / (2 * h)


def invert_vjp(m: O.QGModel, psi_bar: np.ndarray) -> np.ndarray:
    """q_bar = A^T psi_bar with A the (linear) inversion's dense matrix."""
    shape = np.shape(psi_bar)
    n = int(np.prod(shape))
    A = np.empty((n, n))
    e = np.zeros(n)
    for j in range(n):
        e[j] = 1.0
        A[:, j] = O.invert_pv(m, e.reshape(shape)).reshape(-1)
        e[j] = 0.0
    return (A.T @ np.asarray(psi_bar, np.float64).reshape(-1)).reshape(shape)


def integrate(m: O.QGModel, q0: np.ndarray, dt: float, n_steps: int, scheme: str, params: dict | None = None):
    """``qg.integrate`` with parameter overrides (float64)."""
    return O.integrate(m, np.asarray(q0, np.float64), dt, n_steps, scheme, params=_params(m, params))


def fd_directional(loss, x: np.ndarray, d: np.ndarray, rel: float = 1e-4) -> float:
    """Central difference of a scalar loss along d with step rel * |x| / |d|."""
    h = rel * max(float(np.linalg.norm(x)), 1e-300) / max(float(np.linalg.norm(d)), 1e-300)
    return (loss(x + h * d) - loss(x - h * d)) / (2 * h)
