"""The float64 restatement of ReparameterizedQG.project (oracle/reparam.py) against the
reference's own tests of the projection (tests/models/test_qg_reparameterized.py:61-117:
rest state a fixed point, idempotence to discretisation error, finite output, non-zero
geostrophic velocity for a height anomaly) and the operator identity it rests on
(curl of grad_perp = the 5-point Laplacian)."""

import numpy as np

from oracle import qg as O
from oracle import reparam as R


def model(nx=16, ny=16, H=(500.0, 500.0), g_prime=(9.81, 0.02), Lx=4e6, Ly=4e6):
    return O.baroclinic_model(nx=nx, ny=ny, Lx=Lx, Ly=Ly, H=H, g_prime=g_prime)


def rest(m):
    nl, Ny, Nx = m.nl, m.grid.Ny, m.grid.Nx
    return np.ones((nl, Ny, Nx)) * np.asarray(m.H)[:, None, None], np.zeros((nl, Ny, Nx)), np.zeros((nl, Ny, Nx))


def bump(m):
    h, u, v = rest(m)
    h[0, m.grid.Ny // 2, m.grid.Nx // 2] += 1.0
    return h, u, v


def test_rest_state_fixed_point():
    m = model()
    h, u, v = rest(m)
    hg, ug, vg, _ = R.project(m, h, u, v)
    assert np.allclose(hg, h, atol=1e-6)
    assert np.allclose(ug, u, atol=1e-10) and np.allclose(vg, v, atol=1e-10)


def test_idempotent_and_geostrophic():
    m = model()
    p1 = R.project(m, *bump(m))[:3]
    p2 = R.project(m, *p1)[:3]
    for a, b in zip(p2, p1):  # the reference's bound (O(dx^2) at the walls)
        assert np.allclose(a, b, atol=0.1)
    assert np.max(np.abs(p1[1])) > 0 and np.max(np.abs(p1[2])) > 0
    assert all(np.all(np.isfinite(x)) for x in p1)


def test_idempotent_away_from_walls():
    """For a state whose streamfunction vanishes near the walls the projection is exact."""
    m = model(nx=40, ny=36, H=(400.0, 1100.0, 2600.0), g_prime=(9.81, 0.025, 0.0125))
    rng = np.random.default_rng(3)
    psi = np.zeros((3, 38, 42))
    psi[:, 8:-8, 8:-8] = rng.standard_normal((3, 22, 26)) * 1e3
    ug, vg = R.grad_perp(psi, m.grid.dx, m.grid.dy)
    H = np.asarray(m.H)[:, None, None]
    hg = H * (1.0 + m.f0 * m.modes.to_layer(m.modes.eigenvalues[:, None, None] * m.modes.to_modal(psi)))
    h2, u2, v2, psi2 = R.project(m, hg, ug, vg)
    assert np.linalg.norm(psi2 - psi) / np.linalg.norm(psi) < 1e-9
    assert np.linalg.norm(u2 - ug) / np.linalg.norm(ug) < 1e-9
    assert np.linalg.norm((h2 - H) - (hg - H)) / np.linalg.norm(hg - H) < 1e-9


def test_curl_of_grad_perp_is_the_laplacian():
    rng = np.random.default_rng(1)
    psi = rng.standard_normal((2, 20, 24))
    dx, dy = 3.0, 2.0
    z = R.relative_vorticity(*R.grad_perp(psi, dx, dy), dx, dy)
    c = psi[:, 2:-2, 2:-2]
    lap = ((psi[:, 2:-2, 3:-1] + psi[:, 2:-2, 1:-3] - 2 * c) / dx**2
           + (psi[:, 3:-1, 2:-2] + psi[:, 1:-3, 2:-2] - 2 * c) / dy**2)
    assert np.allclose(z[:, 2:-2, 2:-2], lap, rtol=1e-12, atol=1e-12)
