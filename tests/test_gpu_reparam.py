"""ReparameterizedQG.project on the GPU (qg_project through the C ABI: PV kernel, modal DST-I
inversion, reconstruction kernel) against the float64 oracle (oracle/reparam.py), plus the
reference's own properties of the projection (rest-state fixed point, idempotence)."""

import numpy as np
import pytest
import torch

import somax_gb300 as sg
from oracle import qg as O
from oracle import reparam as R
from somax_gb300 import testcases as tc

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = a.detach().cpu().double().numpy() if isinstance(a, torch.Tensor) else a
    b = b.detach().cpu().double().numpy() if isinstance(b, torch.Tensor) else b
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def pair(nx, ny, H, g, Lx=4e6, Ly=3.6e6):
    m = sg.ReparameterizedQG.create(nx=nx, ny=ny, Lx=Lx, Ly=Ly, n_layers=len(H), H=H, g_prime=g)
    o = O.baroclinic_model(nx=nx, ny=ny, Lx=Lx, Ly=Ly, H=H, g_prime=g)
    return m, o


def state(o, seed):
    """A perturbed state: height anomalies of tens of metres and velocities of ~0.1 m/s."""
    nl, Ny, Nx = o.nl, o.grid.Ny, o.grid.Nx
    k = tc.kminus3_field(max(Nx, Ny) - 2, seed, 3 * nl)[:, :Ny, :Nx]
    k = k / np.abs(k).max()
    H = np.asarray(o.H)[:, None, None]
    return H + 20.0 * k[:nl], 0.1 * k[nl:2 * nl], 0.1 * k[2 * nl:]


def cuda(x):
    return torch.tensor(x, dtype=torch.float32, device="cuda")


@pytest.mark.parametrize("nx,ny,H,g", [(16, 16, (500.0, 500.0), (9.81, 0.02)),
                                       (40, 33, (400.0, 1100.0, 2600.0), (9.81, 0.025, 0.0125)),
                                       (128, 128, (400.0, 1100.0, 2600.0), (9.81, 0.025, 0.0125))])
def test_project_against_oracle(nx, ny, H, g):
    m, o = pair(nx, ny, H, g)
    # the oracle sees the FP32-rounded state the GPU sees
    h, u, v = (x.astype(np.float32).astype(np.float64) for x in state(o, 5 + nx))
    got = m.project(sg.MultilayerSW2DState(h=cuda(h), u=cuda(u), v=cuda(v)))
    hg, ug, vg, psi = R.project(o, h, u, v)
    Hb = np.asarray(H)[:, None, None]
    # h_g holds H + anomaly in FP32: the anomaly's floor is half an ulp of H (1.2e-4 m at
    # H = 2600 m against anomalies of metres), hence 3e-5 on it; the velocities difference
    # neighbouring psi values, which magnifies the FP32 inversion's ~1e-6 error of psi (1.6e-5
    # at 130 x 130), hence 5e-5 on them and 1e-5 on psi itself
    assert rel(got.h - torch.tensor(Hb, device="cuda"), hg - Hb) < 3e-5
    assert rel(got.u, ug) < 5e-5
    assert rel(got.v, vg) < 5e-5
    d = m.diagnose(sg.MultilayerSW2DState(h=cuda(h), u=cuda(u), v=cuda(v)))
    assert rel(d.psi, psi) < 1e-5
    assert rel(d.u_ageostrophic, u - ug) < 5e-5


def test_rest_state_and_idempotence():
    m, o = pair(16, 16, (500.0, 500.0), (9.81, 0.02))
    nl, Ny, Nx = 2, 18, 18
    h = cuda(np.ones((nl, Ny, Nx)) * np.asarray([500.0, 500.0])[:, None, None])
    z = torch.zeros_like(h)
    p = m.project(sg.MultilayerSW2DState(h=h, u=z, v=z))
    assert torch.allclose(p.h, h, atol=1e-6) and torch.equal(p.u, z) and torch.equal(p.v, z)
    h[0, Ny // 2, Nx // 2] += 1.0
    p1 = m.project(sg.MultilayerSW2DState(h=h, u=z, v=z))
    p2 = m.project(p1)
    for a, b in ((p2.h, p1.h), (p2.u, p1.u), (p2.v, p1.v)):
        assert torch.allclose(a, b, atol=0.1)
    assert float(p1.u.abs().max()) > 0 and float(p1.v.abs().max()) > 0
    # the second projection against the oracle's projection of the same (FP32) first one: a
    # 1 m bump leaves centimetre anomalies on 500 m, which FP32 holds to a few 1e-4
    r2 = R.project(o, *(x.cpu().double().numpy() for x in (p1.h, p1.u, p1.v)))
    assert rel(p2.u, r2[1]) < 5e-5 and rel(p2.v, r2[2]) < 5e-5


def test_project_rejects_barotropic_and_shapes():
    m, _ = pair(16, 16, (500.0, 500.0), (9.81, 0.02))
    with pytest.raises(ValueError):
        m.project(sg.MultilayerSW2DState(h=torch.zeros(2, 17, 18, device="cuda"),
                                         u=torch.zeros(2, 17, 18, device="cuda"),
                                         v=torch.zeros(2, 17, 18, device="cuda")))
    with pytest.raises(ValueError):
        sg.ReparameterizedQG.create(bc="periodic")


def sw_pair(nx, ny, H, g, Lx=4e6, Ly=3.6e6, nu=200.0, kappa=1e-7, tau=8e-5):
    """The GPU model and the two oracle halves (projection, shallow water) of one basin."""
    from oracle import swm as W

    kw = dict(nx=nx, ny=ny, Lx=Lx, Ly=Ly, n_layers=len(H), H=H, g_prime=g, lateral_viscosity=nu,
              bottom_drag=kappa, wind_amplitude=tau)
    m = sg.ReparameterizedQG.create(**kw)
    o = O.baroclinic_model(nx=nx, ny=ny, Lx=Lx, Ly=Ly, H=H, g_prime=g)
    ms = W.create(nx=nx, ny=ny, Lx=Lx, Ly=Ly, f0=9.375e-5, beta=1.754e-11, H=H, g_prime=g, lateral_viscosity=nu,
                  bottom_drag=kappa, wind_amplitude=tau, bc="wall")
    return m, o, ms


@pytest.mark.parametrize("scheme", ["heun", "tsit5"])
@pytest.mark.parametrize("nx,ny,H,g", [(16, 16, (500.0, 500.0), (9.81, 0.02)),
                                       (40, 33, (400.0, 1100.0, 2600.0), (9.81, 0.025, 0.0125))])
def test_step_matches_oracle(nx, ny, H, g, scheme):
    """10 constant steps of qg_reparam_step (projection + wall rules on every stage input)
    against the float64 composition of the oracle's projection and shallow-water RHS.  One
    projection leaves up to 3e-5 on the h anomaly and 5e-5 on the velocities
    (test_project_against_oracle); 10 steps project 20 (Heun) or 60 (Tsit5) stage inputs.
    Measured on GB300 (h - H, u, v): 16x16 Heun 3.9e-5, 3.1e-5, 4.3e-5; Tsit5 4.5e-5, 6.0e-5,
    6.4e-5; 40x33 Heun 1.7e-4, 4.5e-5, 4.0e-5 (the h anomaly's FP32 storage floor there is
    1.0e-5).  Bounds: 5e-4 on the h anomaly, 1e-4 on the velocities."""
    m, o, ms = sw_pair(nx, ny, H, g)
    h, u, v = (x.astype(np.float32).astype(np.float64) for x in state(o, 3 + nx))
    y0 = np.stack([h, u, v])
    dt = 0.2 * min(o.grid.dx, o.grid.dy) / np.sqrt(9.81 * sum(H))
    got = m.step(sg.MultilayerSW2DState(h=cuda(h), u=cuda(u), v=cuda(v)), dt, 10, scheme)
    assert m.status() == 0
    ref = R.integrate(o, ms, y0, dt, 10, scheme)
    Hb = np.asarray(H)[:, None, None]
    e = (rel(got.h - torch.tensor(Hb, device="cuda"), ref[0] - Hb), rel(got.u, ref[1]), rel(got.v, ref[2]))
    print(f"reparam {nx}x{ny} {scheme}: 10-step rel L2 h-H {e[0]:.2e} u {e[1]:.2e} v {e[2]:.2e}")
    assert e[0] < 5e-4 and max(e[1:]) < 1e-4, e


def test_integrate_and_diagnose_reference_properties():
    """``tests/models/test_qg_reparameterized.py`` on the GPU path: the double-gyre factory
    integrates to finite fields (t1 = 1000 s, dt = 10 s), the rest state stays at rest without
    wind, and diagnose returns finite energies with psi of the state."""
    m, s0 = sg.doublegyre_reparameterized_qg(nx=16, ny=16)
    sol = m.integrate(s0, t0=0.0, t1=1000.0, dt=10.0)
    assert torch.isfinite(sol.ys.h).all() and torch.isfinite(sol.ys.u).all()
    assert float(sol.ys.u.abs().max()) > 0  # the wind spun the top layer up
    m0 = sg.ReparameterizedQG.create(nx=16, ny=16, n_layers=2, H=(500.0, 500.0), g_prime=(9.81, 0.02))
    h = torch.ones((2, 18, 18), device="cuda") * torch.tensor([500.0, 500.0], device="cuda")[:, None, None]
    z = torch.zeros_like(h)
    rest = m0.step(sg.MultilayerSW2DState(h=h, u=z, v=z), 50.0, 5, "tsit5")
    assert torch.allclose(rest.h, h, atol=1e-3) and float(rest.u.abs().max()) < 1e-6
    d = m.diagnose(sol.ys.__class__(h=sol.ys.h[-1], u=sol.ys.u[-1], v=sol.ys.v[-1]))
    assert torch.isfinite(d.total_energy) and (d.energy >= 0).all() and torch.isfinite(d.psi).all()
    assert torch.equal(d.u_ageostrophic, sol.ys.u[-1] - m.project(sg.MultilayerSW2DState(
        h=sol.ys.h[-1], u=sol.ys.u[-1], v=sol.ys.v[-1])).u)
