"""The hand-written adjoint of the multilayer shallow-water model (``qg_swm_rhs_vjp``,
``qg_swm_bc_vjp``, ``qg_swm_step_vjp``; ``somax_gb300/swm_adjoint.py``) against float64
derivatives of the oracle (``oracle/swm.py``: central differences of the restated right-hand
side, exact to O(step^2) where the upwind switch does not flip), and the reference's gradient
test (``tests/models/test_swm_multilayer.py:239-252``).

Tolerances: the VJPs run in FP32 over sums of up to ~40 terms per entry, so 2e-4 relative L2
against the float64 transposed Jacobian; the parameter cotangents (sums over the grid) 1e-4.
"""

import numpy as np
import pytest
import torch

import somax_gb300 as sg
from oracle import swm as W

pytestmark = pytest.mark.gpu


def pair(nx, ny, H, gp, bc, nu=300.0, kappa=1e-5, tau=2e-3):
    kw = dict(nx=nx, ny=ny, Lx=nx * 1e5, Ly=ny * 1e5, f0=1e-4, beta=1.6e-11, H=H, g_prime=gp, lateral_viscosity=nu,
              bottom_drag=kappa, wind_amplitude=tau, bc=bc)
    return sg.MultilayerShallowWater2D.create(n_layers=len(H), **kw), W.create(**kw)


def state(o, seed):
    """A state whose velocities stay away from zero (the upwind switch is not differentiable
    there): u ~ 0.3 + noise, v ~ -0.2 + noise, h ~ H + metres."""
    rng = np.random.default_rng(seed)
    shp = (o.nl, o.Ny, o.Nx)
    h = np.asarray(o.H)[:, None, None] + 3.0 * rng.standard_normal(shp)
    u = 0.3 + 0.05 * rng.standard_normal(shp)
    v = -0.2 + 0.05 * rng.standard_normal(shp)
    return np.stack([h, u, v]).astype(np.float32).astype(np.float64)


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def cuda(x):
    return torch.tensor(np.ascontiguousarray(x), dtype=torch.float32, device="cuda").reshape(-1)


@pytest.mark.parametrize("apply_bc", [True, False])
@pytest.mark.parametrize("bc", ["periodic", "wall"])
@pytest.mark.parametrize("shape", [(5, 4, (500.0, 800.0), (9.81, 0.02)), (6, 7, (400.0,), (9.81,)),
                                   (4, 5, (300.0, 600.0, 900.0), (9.81, 0.03, 0.01))])
def test_rhs_vjp_against_dense_jacobian(shape, bc, apply_bc):
    nx, ny, H, gp = shape
    m, o = pair(nx, ny, H, gp, bc)
    y = state(o, nx + 10 * ny)
    g = np.random.default_rng(7).standard_normal(y.size)
    pl = m.plan()
    yb, pb = pl.rhs_vjp(cuda(y), m._param_vector("cuda"), cuda(g), apply_bc)
    J = W.rhs_jacobian(o, y, apply_bc=apply_bc)
    P = W.rhs_param_derivatives(o, y, apply_bc=apply_bc)
    e_y = rel(yb.cpu().double().numpy(), J.T @ g)
    e_p = np.abs(pb.cpu().double().numpy() - P @ g) / np.maximum(np.abs(P @ g), 1e-30)
    print(f"swm rhs vjp {nx}x{ny}x{len(H)} {bc} apply_bc={apply_bc}: state {e_y:.2e}, params {e_p}")
    assert e_y < 2e-4, e_y
    assert (e_p < 1e-4).all(), e_p


@pytest.mark.parametrize("scheme", ["heun", "ssprk3", "tsit5"])
@pytest.mark.parametrize("bc", ["periodic", "wall"])
def test_step_vjp_against_dense_jacobian(bc, scheme):
    m, o = pair(5, 4, (500.0, 800.0), (9.81, 0.02), bc)
    y = state(o, 3)  # the step continues an integration: no boundary rules on y itself
    dt = 60.0
    g = np.random.default_rng(11).standard_normal(y.size)
    pl = m.plan()
    y0b, pb = pl.step_vjp(cuda(y), m._param_vector("cuda"), dt, scheme, cuda(g))
    J = W.step_jacobian(o, y, dt, 1, scheme)
    e = rel(y0b.cpu().double().numpy(), J.T @ g)
    print(f"swm step vjp {bc} {scheme}: {e:.2e}")
    assert e < 2e-4, e


def test_bc_vjp_is_the_transpose():
    """<B y, g> = <y, B^T g> for the boundary rules, both kinds."""
    for bc in ("periodic", "wall"):
        m, o = pair(6, 5, (500.0, 800.0), (9.81, 0.02), bc)
        rng = np.random.default_rng(1)
        y = rng.standard_normal((3, o.nl, o.Ny, o.Nx))
        g = rng.standard_normal(y.shape)
        By = np.stack(W.apply_boundary_conditions(o, *y))
        gb = m.plan().bc_vjp(cuda(g)).cpu().double().numpy()
        assert abs(np.vdot(By, g) - np.vdot(y.reshape(-1), gb)) < 1e-5 * abs(np.vdot(By, g))


def test_integrate_gradient_against_float64_differences():
    """d loss / d(nu, kappa, tau0) and a directional derivative in h0 through 30 Tsit5 steps
    (checkpoints every 8) against float64 central differences of the oracle integration."""
    m, o = pair(6, 5, (500.0, 800.0), (9.81, 0.02), "wall", nu=200.0, kappa=1e-4, tau=5e-3)
    y0 = state(o, 21)
    dt, n = 60.0, 30
    p = m.params
    m.params = sg.MultilayerSW2DParams(*(torch.tensor(float(x), requires_grad=True)
                                         for x in (p.lateral_viscosity, p.bottom_drag, p.wind_amplitude)))
    h0 = torch.tensor(y0[0], dtype=torch.float32, device="cuda", requires_grad=True)
    s0 = sg.MultilayerSW2DState(h=h0, u=torch.tensor(y0[1], dtype=torch.float32, device="cuda"),
                                v=torch.tensor(y0[2], dtype=torch.float32, device="cuda"))
    sol = m.integrate(s0, 0.0, n * dt, dt, checkpoint_every=8)
    loss = (sol.ys.h[-1].double() ** 2).sum() * 1e-6 + (sol.ys.u[-1].double() ** 2).sum()
    loss.backward()

    def oracle_loss(y, **pp):
        oo = W.create(nx=o.nx, ny=o.ny, Lx=o.Lx, Ly=o.Ly, f0=o.f0, beta=o.beta, H=tuple(o.H),
                      g_prime=tuple(o.g_prime), bc="wall", lateral_viscosity=pp.get("nu", 200.0),
                      bottom_drag=pp.get("kappa", 1e-4), wind_amplitude=pp.get("tau", 5e-3))
        z = W.integrate(oo, y, dt, n, "tsit5")
        return (z[0] ** 2).sum() * 1e-6 + (z[1] ** 2).sum()

    for name, base, got in (("nu", 200.0, m.params.lateral_viscosity.grad),
                            ("kappa", 1e-4, m.params.bottom_drag.grad),
                            ("tau", 5e-3, m.params.wind_amplitude.grad)):
        h = base * 1e-4
        fd = (oracle_loss(y0, **{name: base + h}) - oracle_loss(y0, **{name: base - h})) / (2 * h)
        print(f"swm integrate gradient d/d{name}: {float(got):.6e} vs {fd:.6e}")
        assert abs(float(got) - fd) < 2e-3 * abs(fd), (name, float(got), fd)
    d = np.random.default_rng(5).standard_normal(y0[0].shape)
    eps = 1e-3
    yp, ym = y0.copy(), y0.copy()
    yp[0] += eps * d
    ym[0] -= eps * d
    fd = (oracle_loss(yp) - oracle_loss(ym)) / (2 * eps)
    got = float((h0.grad.cpu().double().numpy() * d).sum())
    print(f"swm integrate gradient, h0 direction: {got:.6e} vs {fd:.6e}")
    assert abs(got - fd) < 2e-3 * abs(fd)


def test_reference_grad_through_params():
    """``test_swm_multilayer.py:239-252``: a 0.1 m bump on the rest state, 50 one-second steps,
    loss sum(h^2): the lateral viscosity's gradient is finite."""
    m = sg.MultilayerShallowWater2D.create(nx=16, ny=16, n_layers=2, H=(500.0, 500.0), g_prime=(9.81, 0.02),
                                           lateral_viscosity=100.0)
    m.params = sg.MultilayerSW2DParams(torch.tensor(100.0, requires_grad=True), torch.tensor(0.0),
                                       torch.tensor(0.0))
    Ny, Nx = m.grid.Ny, m.grid.Nx
    h0 = torch.ones((2, Ny, Nx), device="cuda") * torch.tensor([500.0, 500.0], device="cuda")[:, None, None]
    h0[0, Ny // 2, Nx // 2] += 0.1
    z = torch.zeros_like(h0)
    sol = m.integrate(sg.MultilayerSW2DState(h=h0, u=z, v=z), t0=0.0, t1=50.0, dt=1.0)
    loss = (sol.ys.h.double() ** 2).sum()
    loss.backward()
    assert torch.isfinite(m.params.lateral_viscosity.grad)
