"""Masked basins in the oracle (test infrastructure only): a land mask on T-cells and the
capacitance-matrix correction of the DST-I Helmholtz solve.

An extension: somax's live code has no land mask (the capacitance solver appears only in its
historical notebooks, ``notebooks/dev/QG_Multilayer``, importing deleted modules).  The
method restated is the capacitance-matrix method for a DST-I solver on an irregular domain
(Thiry et al. 2024, the MQGeometry paper the reference's notes cite).  No reference output
exists for it: parity of the masked path is unpinned, and this module checks the GPU's
capacitance correction against a direct sparse solve of the same discrete problem.

Semantics (the ring keeps the unmasked model's rules; ``land`` = mask == 0 on interior cells):
  * q reads as 0 on land;
  * B = land cells with an interior ocean cell among their 8 neighbours (every cell the
    ocean's 9-point Arakawa and 5-point stencils reach);
  * the Helmholtz problem per mode: (lap - lam) psi = rhs at every cell outside B (the full
    array, zeros outside it, as ``qg.helmholtz_dst``) and psi = 0 on B;
  * psi is then zero on all land (and on the ring for the baroclinic model);
  * lap(q) is zero on land (as on the ring), and dq is zero on land.
With no land this is exactly the unmasked model.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import qg as O


def land(mask: np.ndarray) -> np.ndarray:
    """Interior land cells (bool, Ny x Nx); the ring is never land."""
    m = np.asarray(mask) == 0
    m = m.copy()
    m[0, :] = m[-1, :] = m[:, 0] = m[:, -1] = False
    return m


def boundary_points(mask: np.ndarray) -> np.ndarray:
    """Linear indices (j * Nx + i, ascending) of B: land cells with an interior ocean cell
    among their 8 neighbours."""
    L = land(mask)
    ocean = ~L
    ocean[0, :] = ocean[-1, :] = ocean[:, 0] = ocean[:, -1] = False
    Ny, Nx = L.shape
    near = np.zeros_like(L)
    p = np.pad(ocean, 1)
    for dj in (-1, 0, 1):
        for di in (-1, 0, 1):
            if dj or di:
                near |= p[1 + dj:1 + dj + Ny, 1 + di:1 + di + Nx]
    return np.flatnonzero((L & near).reshape(-1))


def _operator(Ny: int, Nx: int, dx: float, dy: float, lam: float) -> sp.csr_matrix:
    """Full-array 5-point (lap - lam) with zeros outside the array (the DST-I operator)."""
    def d2(n, d):
        e = np.ones(n)
        return sp.diags([e[:-1], -2 * e, e[:-1]], [-1, 0, 1]) / d**2
    return (sp.kron(sp.identity(Ny), d2(Nx, dx)) + sp.kron(d2(Ny, dy), sp.identity(Nx))
            - lam * sp.identity(Ny * Nx)).tocsr()


_LU_CACHE: dict = {}


def _factor(mask: np.ndarray, dx: float, dy: float, lam: float):
    """Sparse LU of the masked operator (B rows replaced by the identity), cached per mask,
    spacing and lambda (a time loop reuses it)."""
    m = np.ascontiguousarray(mask, dtype=np.uint8)
    key = (m.shape, hash(m.tobytes()), float(dx), float(dy), float(lam))
    if key not in _LU_CACHE:
        Ny, Nx = m.shape
        A = _operator(Ny, Nx, dx, dy, lam).tolil()
        B = boundary_points(m)
        for k in B:
            A.rows[k] = [k]
            A.data[k] = [1.0]
        if len(_LU_CACHE) > 16:
            _LU_CACHE.clear()
        _LU_CACHE[key] = (spla.splu(A.tocsc()), B)
    return _LU_CACHE[key]


def helmholtz_masked(rhs: np.ndarray, dx: float, dy: float, lam: float, mask: np.ndarray) -> np.ndarray:
    """Direct sparse solve: (lap - lam) psi = rhs off B, psi = 0 on B (float64)."""
    Ny, Nx = rhs.shape
    lu, B = _factor(mask, dx, dy, lam)
    b = np.asarray(rhs, np.float64).reshape(-1).copy()
    b[B] = 0.0
    return lu.solve(b).reshape(Ny, Nx)


def capacitance_matrix(Ny: int, Nx: int, dx: float, dy: float, lam: float, B: np.ndarray) -> np.ndarray:
    """C = G[B, B] with G the unmasked DST-I solve (columns from unit sources)."""
    k = len(B)
    C = np.empty((k, k))
    e = np.zeros(Ny * Nx)
    for c, b in enumerate(B):
        e[b] = 1.0
        C[:, c] = O.helmholtz_dst(e.reshape(Ny, Nx), dx, dy, lam).reshape(-1)[B]
        e[b] = 0.0
    return C


def helmholtz_capacitance(rhs: np.ndarray, dx: float, dy: float, lam: float, mask: np.ndarray) -> np.ndarray:
    """The capacitance-matrix method: psi1 = G rhs0 (rhs0 = rhs with B zeroed),
    sigma = -C^-1 psi1[B], psi = G(rhs0 + E_B sigma); psi is 0 on B and solves the equation
    everywhere else."""
    Ny, Nx = rhs.shape
    B = boundary_points(mask)
    r0 = np.asarray(rhs, np.float64).reshape(-1).copy()
    r0[B] = 0.0
    r0 = r0.reshape(Ny, Nx)
    psi1 = O.helmholtz_dst(r0, dx, dy, lam)
    if len(B) == 0:
        return psi1
    C = capacitance_matrix(Ny, Nx, dx, dy, lam, B)
    sigma = -np.linalg.solve(C, psi1.reshape(-1)[B])
    r2 = r0.reshape(-1).copy()
    r2[B] += sigma
    return O.helmholtz_dst(r2.reshape(Ny, Nx), dx, dy, lam)


def invert_pv(m: O.QGModel, q: np.ndarray, mask: np.ndarray) -> np.ndarray:
    """psi of a masked member: per-mode masked Helmholtz (direct sparse solve), to layers,
    zero on land (and on the ring for the baroclinic model)."""
    g = m.grid
    L = land(mask)
    q = np.where(L, 0.0, np.asarray(q, np.float64))
    if m.barotropic:
        psi = helmholtz_masked(q, g.dx, g.dy, 0.0, mask)
        return np.where(L, 0.0, psi)
    qm = m.modes.to_modal(q)
    lam = m.helmholtz_lambdas
    pm = np.stack([helmholtz_masked(qm[k], g.dx, g.dy, float(lam[k]), mask) for k in range(m.nl)])
    psi = O.zero_boundaries(m.modes.to_layer(pm))
    return np.where(L, 0.0, psi)


def vector_field(m: O.QGModel, q: np.ndarray, mask: np.ndarray, params: dict | None = None) -> np.ndarray:
    """dq/dt of a masked member (``qg.vector_field`` with the land rules above)."""
    p = dict(lateral_viscosity=m.lateral_viscosity, bottom_drag=m.bottom_drag,
             wind_amplitude=m.wind_amplitude, biharmonic_viscosity=m.biharmonic_viscosity)
    if params:
        p.update(params)
    g = m.grid
    L = land(mask)
    q = np.where(L, 0.0, np.asarray(q, np.float64))
    psi = invert_pv(m, q, mask)
    by = m.beta_y()
    F = m.wind_forcing()
    lq = np.where(L, 0.0, O.laplacian(q, g.dx, g.dy))
    if m.barotropic:
        dq = np.zeros_like(q)
        dq[1:-1, 1:-1] = -O.arakawa_jacobian(psi, q + by, g.dx, g.dy)
        dq = dq + p["wind_amplitude"] * F
        dq = dq - p["bottom_drag"] * O.laplacian(psi, g.dx, g.dy)
    else:
        dq = np.zeros_like(q)
        dq[:, 1:-1, 1:-1] = -O.arakawa_jacobian(psi, q + by[None], g.dx, g.dy)
        dq[0] = dq[0] + p["wind_amplitude"] * F / m.H[0]
        dq[-1] = dq[-1] - p["bottom_drag"] * O.laplacian(psi[-1], g.dx, g.dy)
    dq = dq + p["lateral_viscosity"] * lq
    if p["biharmonic_viscosity"] != 0:
        dq = dq - p["biharmonic_viscosity"] * O.laplacian(lq, g.dx, g.dy)
    return np.where(L, 0.0, dq)


def integrate(m: O.QGModel, q0: np.ndarray, mask: np.ndarray, dt: float, n_steps: int, scheme: str = "ssprk3"):
    """``qg.integrate`` for a masked member: BC (ring and land) on the initial state, BC on
    every stage input."""

    def f(y):
        return vector_field(m, O.apply_boundary_conditions(m, y), mask)

    y = np.where(land(mask), 0.0, O.apply_boundary_conditions(m, np.asarray(q0, np.float64)))
    for _ in range(n_steps):
        y = O.rk_step(f, y, dt, scheme)
    return y


def helmholtz_residual(psi: np.ndarray, rhs: np.ndarray, dx: float, dy: float, lam: float,
                       mask: np.ndarray) -> float:
    """|| rhs - (lap - lam) psi ||  /  || rhs || over the cells off B (the equations solved)."""
    r = np.asarray(rhs, np.float64) - O.helmholtz_apply_full(np.asarray(psi, np.float64), dx, dy, lam)
    keep = np.ones(r.size, bool)
    keep[boundary_points(mask)] = False
    return float(np.linalg.norm(r.reshape(-1)[keep]) / max(np.linalg.norm(np.asarray(rhs).reshape(-1)[keep]), 1e-300))
