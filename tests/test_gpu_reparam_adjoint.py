"""The reverse mode of ReparameterizedQG (``qg_project_vjp``, ``qg_reparam_bc_vjp``,
``qg_reparam_step_vjp`` through ``somax_gb300.swm_adjoint.Integrate``) against float64
differences of the oracle (``oracle/reparam.py`` composed with ``oracle/swm.py``), and the
reference's gradient test (``tests/models/test_qg_reparameterized.py:193-206``).

The projection is affine, so the columns of its linear part are exact differences of two oracle
projections.  The FP32 inversion inside the projection (~1e-6 relative) bounds the agreement:
1e-4 relative L2.  Measured on GB300: step VJPs 1.7e-7 (Heun) and 5.5e-7 (Tsit5) against the
float64 transposed Jacobian; 12-step gradients in nu, kappa, tau0 within 5e-5 of float64
differences."""

import numpy as np
import pytest
import torch

import somax_gb300 as sg
from oracle import qg as O
from oracle import reparam as R
from oracle import swm as W

pytestmark = pytest.mark.gpu


def models(nx, ny, H, gp, nu=200.0, kappa=1e-4, tau=5e-3):
    kw = dict(nx=nx, ny=ny, Lx=nx * 1e5, Ly=ny * 1e5, n_layers=len(H), H=H, g_prime=gp, lateral_viscosity=nu,
              bottom_drag=kappa, wind_amplitude=tau)
    m = sg.ReparameterizedQG.create(**kw)
    o = O.baroclinic_model(nx=nx, ny=ny, Lx=nx * 1e5, Ly=ny * 1e5, H=H, g_prime=gp)
    ms = W.create(nx=nx, ny=ny, Lx=nx * 1e5, Ly=ny * 1e5, f0=9.375e-5, beta=1.754e-11, H=H, g_prime=gp,
                  lateral_viscosity=nu, bottom_drag=kappa, wind_amplitude=tau, bc="wall")
    return m, o, ms


def state(o, seed):
    rng = np.random.default_rng(seed)
    shp = (o.nl, o.grid.Ny, o.grid.Nx)
    h = np.asarray(o.H)[:, None, None] + 3.0 * rng.standard_normal(shp)
    u = 0.3 + 0.05 * rng.standard_normal(shp)
    v = -0.2 + 0.05 * rng.standard_normal(shp)
    return np.stack([h, u, v]).astype(np.float32).astype(np.float64)


def cuda(x):
    return torch.tensor(np.ascontiguousarray(x), dtype=torch.float32, device="cuda").reshape(-1)


def test_project_vjp_against_dense_transpose():
    """qg_project_vjp against the float64 transpose of the projection's linear part, whose
    columns are differences of two oracle projections (the projection is affine)."""
    import ctypes as C

    from somax_gb300 import _lib
    from somax_gb300.qg import _stream_handle

    m, o, _ = models(8, 6, (500.0, 800.0, 1500.0), (9.81, 0.025, 0.0125))
    y = state(o, 1)
    base = np.stack(R.project(o, *y)[:3]).reshape(-1)
    n = y.size
    L = np.empty((n, n))
    flat = y.reshape(-1)
    for c in range(n):
        z = flat.copy()
        z[c] += 1.0
        L[:, c] = np.stack(R.project(o, *z.reshape(y.shape))[:3]).reshape(-1) - base
    g = np.random.default_rng(2).standard_normal(n)
    qp = m.plan()
    gd = cuda(g)
    out = torch.empty_like(gd)
    lay, f = gd.numel() // 3, 4
    a, b = int(gd.data_ptr()), int(out.data_ptr())
    _lib.check(qp._L.qg_project_vjp(qp._h, C.c_void_p(a), C.c_void_p(a + lay * f), C.c_void_p(a + 2 * lay * f),
                                    C.c_void_p(b), C.c_void_p(b + lay * f), C.c_void_p(b + 2 * lay * f),
                                    _stream_handle(gd.device)), "qg_project_vjp")
    ref = L.T @ g
    e = float(np.linalg.norm(out.cpu().double().numpy() - ref) / np.linalg.norm(ref))
    print(f"project vjp against the dense transpose: {e:.2e}")
    assert e < 1e-4, e


@pytest.mark.parametrize("scheme", ["heun", "tsit5"])
def test_reparam_step_vjp_against_dense_jacobian(scheme):
    m, o, ms = models(5, 4, (500.0, 800.0), (9.81, 0.02))
    y = state(o, 3)
    dt = 60.0

    def bc(z):
        return np.stack(R.project(o, *W.apply_boundary_conditions(ms, z[0], z[1], z[2]))[:3])

    def step(z):
        return O.rk_step(lambda w: np.stack(W.vector_field(ms, *bc(w))), z, dt, scheme)

    n = y.size
    flat = y.reshape(-1)
    scale = [max(np.abs(y[f]).max(), 1e-3) * 1e-6 for f in range(3)]
    J = np.empty((n, n))
    for c in range(n):
        h = scale[c // (n // 3)]
        yp, ym = flat.copy(), flat.copy()
        yp[c] += h
        ym[c] -= h
        J[:, c] = (step(yp.reshape(y.shape)) - step(ym.reshape(y.shape))).reshape(-1) / (2 * h)
    g = np.random.default_rng(4).standard_normal(n)
    from somax_gb300.reparameterized import _ReparamStepper

    st = _ReparamStepper(m, torch.device("cuda"))
    yb, _ = st.step_vjp(cuda(y), m.swm._param_vector("cuda"), dt, scheme, cuda(g))
    ref = J.T @ g
    e = float(np.linalg.norm(yb.cpu().double().numpy() - ref) / np.linalg.norm(ref))
    print(f"reparam step vjp {scheme}: {e:.2e}")
    assert e < 1e-4, e


def test_reparam_integrate_gradient_against_float64_differences():
    m, o, ms = models(8, 6, (500.0, 800.0), (9.81, 0.02))
    y0 = state(o, 9)
    dt, n = 60.0, 12
    p = m.params
    m.params = sg.MultilayerSW2DParams(*(torch.tensor(float(x), requires_grad=True)
                                         for x in (p.lateral_viscosity, p.bottom_drag, p.wind_amplitude)))
    s0 = sg.MultilayerSW2DState(*(torch.tensor(y0[k], dtype=torch.float32, device="cuda") for k in range(3)))
    sol = m.integrate(s0, 0.0, n * dt, dt, checkpoint_every=5)
    loss = (sol.ys.u[-1].double() ** 2).sum() + (sol.ys.v[-1].double() ** 2).sum()
    loss.backward()

    def oracle_loss(nu=200.0, kappa=1e-4, tau=5e-3):
        ms2 = W.create(nx=8, ny=6, Lx=8e5, Ly=6e5, f0=9.375e-5, beta=1.754e-11, H=(500.0, 800.0), g_prime=(9.81, 0.02),
                       lateral_viscosity=nu, bottom_drag=kappa, wind_amplitude=tau, bc="wall")
        z = R.integrate(o, ms2, y0, dt, n, "tsit5")
        return (z[1] ** 2).sum() + (z[2] ** 2).sum()

    for name, base, got in (("nu", 200.0, m.params.lateral_viscosity.grad),
                            ("kappa", 1e-4, m.params.bottom_drag.grad),
                            ("tau", 5e-3, m.params.wind_amplitude.grad)):
        h = base * 1e-4
        fd = (oracle_loss(**{name: base + h}) - oracle_loss(**{name: base - h})) / (2 * h)
        print(f"reparam integrate gradient d/d{name}: {float(got):.6e} vs {fd:.6e}")
        assert abs(float(got) - fd) < 2e-3 * abs(fd), (name, float(got), fd)


def test_reference_grad_through_params():
    """``test_qg_reparameterized.py:190-206``: a 0.1 m bump on the rest state of a 2-layer 16^2
    basin, 50 one-second steps, loss sum(h^2): the lateral viscosity's gradient is finite."""
    m = sg.ReparameterizedQG.create(nx=16, ny=16, n_layers=2, H=(500.0, 500.0), g_prime=(9.81, 0.02),
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
