"""The test-case factories of ``somax/_src/models/gfd_testcases.py`` (somax_gb300.gfd_testcases):
types, shapes and initial fields on the host; the GPU integrations of
``tests/models/test_gfd_testcases.py``, ``test_qg_baroclinic.py:315-326``,
``test_qg_reparameterized.py:209-220`` and ``test_swm_multilayer.py:255-265``."""

import math

import numpy as np
import pytest
import torch

import somax_gb300 as sg


def test_factories_types_and_shapes():
    m, s = sg.doublegyre_qg(nx=16, ny=16, device="cpu")
    assert isinstance(m, sg.BarotropicQG) and isinstance(s, sg.BarotropicQGState)
    assert s.q.shape == (m.grid.Ny, m.grid.Nx) and float(s.q.abs().max()) == 0.0
    assert float(m.params.wind_amplitude) == pytest.approx(1e-12) and m.consts.f0 == 1e-4
    m, s = sg.doublegyre_baroclinic_qg(nx=16, ny=16, device="cpu")
    assert isinstance(m, sg.BaroclinicQG) and isinstance(s, sg.BaroclinicQGState)
    assert s.q.shape == (3, 18, 18) and m.consts.n_layers == 3
    assert float(m.params.wind_amplitude) == pytest.approx(1.3e-10) and float(m.params.lateral_viscosity) == 15.0
    m, s = sg.doublegyre_reparameterized_qg(nx=16, ny=16, device="cpu")
    assert isinstance(m, sg.ReparameterizedQG) and isinstance(s, sg.MultilayerSW2DState)
    assert s.h.shape[0] == 3 and torch.equal(s.h[:, 5, 7], torch.tensor([400.0, 1100.0, 2600.0]))
    assert m.swm.bc_type == "wall" and float(m.params.bottom_drag) == pytest.approx(3.6e-8)
    m, s = sg.baroclinic_instability_swm(nx=16, ny=16, device="cpu")
    assert isinstance(m, sg.MultilayerShallowWater2D) and m.bc_type == "periodic"
    assert s.h.shape[0] == 2 and torch.equal(s.h[:, 0, 0], torch.tensor([500.0, 4500.0]))


def test_barotropic_jet_factory():
    """gfd_testcases.py:121-181: one periodic layer of depth H0, the Gaussian jet in u and the
    sin(4 pi x / Lx) perturbation in v."""
    m, s = sg.barotropic_jet_instability(nx=32, ny=32, device="cpu")
    assert isinstance(m, sg.NonlinearShallowWater2D) and isinstance(s, sg.NonlinearSW2DState)
    assert s.h.shape == (34, 34) and float(s.h.min()) == float(s.h.max()) == 1000.0
    g = m.grid
    env = np.exp(-0.5 * ((np.arange(g.Ny) * g.dy - g.Ly / 2) / 5e4) ** 2)
    assert np.allclose(s.u[:, 5].double().numpy(), env, rtol=1e-6, atol=1e-9)
    assert m.consts.H0 == 1000.0 and m.swm.bc_type == "periodic"


def test_jet_fields():
    """Opposite Gaussian jets about Ly / 2 and a sin(4 pi x / Lx) perturbation under the same
    envelope (gfd_testcases.py:344-359), on the padded grid (x_i = i dx, y_j = j dy)."""
    m, s = sg.baroclinic_instability_swm(nx=32, ny=32, device="cpu")
    g = m.grid
    assert torch.allclose(s.u[0], -s.u[1])
    y = np.arange(g.Ny) * g.dy
    x = np.arange(g.Nx) * g.dx
    env = np.exp(-0.5 * ((y - g.Ly / 2) / 5e4) ** 2)
    assert np.allclose(s.u[0, :, 3].double().numpy(), 0.5 * env, rtol=1e-6, atol=1e-9)
    want_v = 0.01 * np.sin(4 * math.pi * x / g.Lx)[None, :] * env[:, None]
    assert np.allclose(s.v[1].double().numpy(), want_v, rtol=1e-5, atol=1e-10)
    assert torch.equal(s.v[0], s.v[1])


@pytest.mark.gpu
def test_factories_integrate_finite_on_gpu():
    m, s = sg.doublegyre_qg(nx=16, ny=16)
    assert torch.isfinite(m.integrate(s, t0=0.0, t1=100.0, dt=1.0).ys.q).all()
    m, s = sg.doublegyre_baroclinic_qg(nx=16, ny=16)
    sol = m.integrate(s, t0=0.0, t1=3600.0, dt=100.0)
    assert torch.isfinite(sol.ys.q).all() and float(sol.ys.q.abs().max()) > 0
    m, s = sg.baroclinic_instability_swm(nx=16, ny=16)
    sol = m.integrate(s, t0=0.0, t1=1000.0, dt=10.0)
    assert torch.isfinite(sol.ys.h).all() and m.status() == 0
