"""``NonlinearShallowWater2D`` (``swm/nonlinear_2d.py``) on the multilayer engine: the one-layer
case with g' = g and the wind not divided by the depth, against the float64 restatement
(``oracle/swm.py`` with H = (1,), which enters only that division), and the reference's own
tests of the model (``tests/models/test_swm_2d.py:126-174``) and of ``barotropic_jet_instability``
(``tests/models/test_gfd_testcases.py:57-68``)."""

import numpy as np
import pytest
import torch

import somax_gb300 as sg
from oracle import swm as W

pytestmark = pytest.mark.gpu


def pair(nx, ny, bc, H0=100.0, nu=300.0, kappa=1e-5, tau=2e-5, Lx=1.2e6, Ly=0.9e6):
    m = sg.NonlinearShallowWater2D.create(nx=nx, ny=ny, Lx=Lx, Ly=Ly, f0=1e-4, beta=1.6e-11, H0=H0,
                                          lateral_viscosity=nu, bottom_drag=kappa, wind_amplitude=tau, bc=bc)
    o = W.create(nx=nx, ny=ny, Lx=Lx, Ly=Ly, f0=1e-4, beta=1.6e-11, H=(1.0,), g_prime=(9.81,),
                 lateral_viscosity=nu, bottom_drag=kappa, wind_amplitude=tau, bc=bc)
    return m, o


def state(o, seed, H0=100.0):
    rng = np.random.default_rng(seed)
    shp = (o.Ny, o.Nx)
    h = H0 + 2.0 * rng.standard_normal(shp)
    u = 0.2 * rng.standard_normal(shp)
    v = 0.2 * rng.standard_normal(shp)
    return np.stack([h, u, v]).astype(np.float32).astype(np.float64)


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def gpu_state(y):
    return sg.NonlinearSW2DState(*(torch.tensor(y[k], dtype=torch.float32, device="cuda") for k in range(3)))


@pytest.mark.parametrize("bc", ["periodic", "wall"])
def test_rhs_and_steps_match_oracle(bc):
    m, o = pair(23, 17, bc)
    y = state(o, 3)
    t = m.vector_field(0.0, gpu_state(y))
    ref = W.vector_field(o, y[0][None], y[1][None], y[2][None])
    f32 = W.vector_field(o, *(y[k][None].astype(np.float32) for k in range(3)))
    for k, g in enumerate((t.h, t.u, t.v)):
        tol = max(2e-5, 4 * rel(f32[k][0], ref[k][0]))
        assert rel(g.cpu().double().numpy(), ref[k][0]) < tol, (k, tol)
    dt = 0.2 * min(o.dx, o.dy) / np.sqrt(9.81 * 100.0)
    got = m.step(gpu_state(y), dt, 20, "tsit5")
    ref = W.integrate(o, y[:, None], dt, 20, "tsit5")[:, 0]
    f32 = W.integrate(o, y[:, None].astype(np.float32), dt, 20, "tsit5")[:, 0]
    assert m.status() == 0
    for k, g in enumerate((got.h, got.u, got.v)):
        tol = max(1e-5, 4 * rel(f32[k], ref[k]))
        assert rel(g.cpu().double().numpy(), ref[k]) < tol, (k, tol)


def _gaussian_state(m, amp=0.1):
    g = m.grid
    x = torch.arange(g.Nx, dtype=torch.float64) * g.dx
    y = torch.arange(g.Ny, dtype=torch.float64) * g.dy
    Y, X = torch.meshgrid(y, x, indexing="ij")
    bump = torch.exp(-0.5 * (((X - g.Lx / 2) / (g.Lx / 5)) ** 2 + ((Y - g.Ly / 2) / (g.Lx / 5)) ** 2))
    h0 = (100.0 + amp * bump).to(device="cuda", dtype=torch.float32)
    return sg.NonlinearSW2DState(h=h0, u=torch.zeros_like(h0), v=torch.zeros_like(h0))


def test_reference_properties():
    """test_swm_2d.py: a 0.1 m Gaussian bump integrates to finite fields (t1 = 10 s, dt = 0.1 s),
    diagnose gives PV and vorticity of the state's shape, and the lateral viscosity's gradient
    through integrate (t1 = 5 s, loss sum(h^2)) is finite."""
    m = sg.NonlinearShallowWater2D.create(nx=16, ny=16, H0=100.0, lateral_viscosity=100.0)
    s0 = _gaussian_state(m)
    sol = m.integrate(s0, t0=0.0, t1=10.0, dt=0.1)
    assert torch.isfinite(sol.ys.h).all() and sol.ys.h.shape[-2:] == (18, 18)
    d = m.diagnose(sg.NonlinearSW2DState(h=s0.h, u=s0.u, v=s0.v))
    assert d.potential_vorticity.shape == s0.h.shape and d.relative_vorticity.shape == s0.h.shape
    assert torch.isfinite(d.energy) and d.energy.dim() == 0
    m.params = sg.NonlinearSW2DParams(torch.tensor(100.0, requires_grad=True), torch.tensor(0.0), torch.tensor(0.0))
    rest = sg.NonlinearSW2DState(h=torch.full_like(s0.h, 100.0), u=torch.zeros_like(s0.h), v=torch.zeros_like(s0.h))
    loss = (m.integrate(rest, t0=0.0, t1=5.0, dt=0.1).ys.h.double() ** 2).sum()
    loss.backward()
    assert torch.isfinite(m.params.lateral_viscosity.grad)


def test_barotropic_jet_instability_integrates():
    m, s0 = sg.barotropic_jet_instability(nx=32, ny=32)
    sol = m.integrate(s0, t0=0.0, t1=100.0, dt=1.0)
    assert torch.isfinite(sol.ys.h).all() and m.status() == 0
