"""The float64 shallow-water restatement (``oracle/swm.py``) on CPU: the reference's own tests
of ``MultilayerShallowWater2D`` (``tests/models/test_swm_multilayer.py``) restated on it, plus
the conservation properties the C-grid operators give."""

import numpy as np
import pytest

from oracle import qg as Q
from oracle import swm as W


def model(**kw):
    d = dict(nx=16, ny=16, H=(500.0, 500.0), g_prime=(9.81, 0.02))
    d.update(kw)
    return W.create(**d)


def rest(m):
    h = np.ones((m.nl, m.Ny, m.Nx)) * m.H[:, None, None]
    return h, np.zeros_like(h), np.zeros_like(h)


def bumped(m, amp=1.0):
    h, u, v = rest(m)
    h[0, m.Ny // 2, m.Nx // 2] += amp
    return h, u, v


def test_create_validation():
    with pytest.raises(ValueError):
        W.create(nx=16, ny=16, H=(500.0, 500.0), g_prime=(9.81, 0.02, 0.01))


@pytest.mark.parametrize("bc", ["periodic", "wall"])
def test_rest_state_zero_tendency(bc):
    m = model(bc=bc)
    t = W.vector_field(m, *W.apply_boundary_conditions(m, *rest(m)))
    assert max(np.abs(x).max() for x in t) < 1e-10


def test_wind_forcing_top_layer_only():
    m = model(wind_amplitude=1e-5)
    _, du, _ = W.vector_field(m, *W.apply_boundary_conditions(m, *rest(m)))
    assert np.abs(du[0]).max() > 0 and np.abs(du[-1]).max() < 1e-15


def test_bottom_drag_bottom_layer_only():
    m = model(bottom_drag=1e-4)
    h, u, v = rest(m)
    u[:] = 1.0
    _, du, _ = W.vector_field(m, *W.apply_boundary_conditions(m, h, u, v))
    assert np.all(np.isfinite(du))
    # uniform flow: everything but the drag cancels in the interior of the bottom layer
    assert np.allclose(du[-1][1:-1, 1:-1] - du[0][1:-1, 1:-1], -1e-4, rtol=0, atol=1e-12)


def test_pressure_coupling_between_layers():
    m = model()
    _, du, _ = W.vector_field(m, *W.apply_boundary_conditions(m, *bumped(m)))
    assert np.abs(du[1]).max() > 0


def test_wall_bcs():
    m = model(bc="wall")
    h, u, v = rest(m)
    u[:] = 1.0
    v[:] = 1.0
    h2, u2, v2 = W.apply_boundary_conditions(m, h + np.random.default_rng(0).standard_normal(h.shape), u, v)
    assert np.allclose(u2[:, :, 0], 0) and np.allclose(u2[:, :, -1], 0) and np.allclose(u2[:, :, -2], 0)
    assert np.allclose(v2[:, 0, :], 0) and np.allclose(v2[:, -1, :], 0) and np.allclose(v2[:, -2, :], 0)
    assert np.array_equal(h2[:, 0, 1:-1], h2[:, 1, 1:-1]) and np.array_equal(h2[:, 1:-1, -1], h2[:, 1:-1, -2])


def test_periodic_bcs_wrap():
    m = model(bc="periodic")
    r = np.random.default_rng(1).standard_normal((m.nl, m.Ny, m.Nx))
    h2, _, _ = W.apply_boundary_conditions(m, r, r, r)
    assert np.array_equal(h2[:, 0, :], h2[:, -2, :]) and np.array_equal(h2[:, :, -1], h2[:, :, 1])


@pytest.mark.parametrize("bc", ["periodic", "wall"])
def test_mass_conserved(bc):
    """The flux-form upwind mass equation conserves sum(h) over the interior to rounding."""
    m = model(bc=bc, lateral_viscosity=100.0)
    rng = np.random.default_rng(2)
    h, u, v = bumped(m, 5.0)
    u += 0.3 * rng.standard_normal(u.shape)
    v += 0.3 * rng.standard_normal(v.shape)
    h, u, v = W.apply_boundary_conditions(m, h, u, v)
    dh, _, _ = W.vector_field(m, h, u, v)
    s = (Ellipsis, slice(1, -1), slice(1, -1))
    if bc == "wall":
        assert abs(dh[s].sum()) < 1e-9 * np.abs(dh[s]).sum()
    else:
        # periodic: what leaves through the east / north faces comes back through the west / south
        assert abs(dh[s].sum()) < 1e-9 * np.abs(dh[s]).sum()


@pytest.mark.parametrize("nl", [2, 3])
def test_integrate_short_is_finite(nl):
    H, gp = ((500.0, 500.0), (9.81, 0.02)) if nl == 2 else ((400.0, 1100.0, 2500.0), (9.81, 0.025, 0.0125))
    m = W.create(nx=16, ny=16, H=H, g_prime=gp, lateral_viscosity=100.0)
    y0 = np.stack(bumped(m))
    y = W.integrate(m, y0, 10.0, 100, "tsit5")
    assert np.all(np.isfinite(y))


def test_energy_nonnegative_and_diagnose_shapes():
    m = model()
    d = W.diagnose(m, *rest(m))
    assert np.all(d["energy"] >= 0)
    assert d["potential_vorticity"].shape == (2, m.Ny, m.Nx)
    assert np.isfinite(d["total_energy"]) and np.isfinite(d["total_enstrophy"])


def test_float32_restatement_close_to_float64():
    """The restatement is dtype-generic: run in float32 it stays within FP32 rounding of the
    float64 run (what the GPU comparisons use as their floor)."""
    m = model(lateral_viscosity=100.0, wind_amplitude=1e-5, bc="wall", beta=1.6e-11)
    rng = np.random.default_rng(3)
    h, u, v = bumped(m, 3.0)
    u += 0.2 * rng.standard_normal(u.shape)
    v += 0.2 * rng.standard_normal(v.shape)
    y = np.stack(W.apply_boundary_conditions(m, h, u, v))
    a = W.rhs(m, y)
    b = W.rhs(m, y.astype(np.float32))
    assert b.dtype == np.float32
    for k in range(3):
        assert np.linalg.norm(b[k] - a[k]) / np.linalg.norm(a[k]) < 1e-4


def test_oracle_derivatives_are_consistent():
    """The float64 derivatives the adjoint tests use (test infrastructure): the dense
    Jacobian applied to a direction equals a central difference along it, and the parameter
    derivatives (the right-hand side is affine in each) equal differences of any step."""
    import numpy as np

    from oracle import swm as W

    m = W.create(nx=5, ny=4, Lx=5e5, Ly=4e5, f0=1e-4, beta=1.6e-11, H=(500.0, 800.0), g_prime=(9.81, 0.02),
                 lateral_viscosity=300.0, bottom_drag=1e-5, wind_amplitude=2e-3, bc="wall")
    rng = np.random.default_rng(0)
    y = np.stack([np.asarray(m.H)[:, None, None] + rng.standard_normal((2, 6, 7)),
                  0.3 + 0.1 * rng.standard_normal((2, 6, 7)), -0.2 + 0.1 * rng.standard_normal((2, 6, 7))])
    J = W.rhs_jacobian(m, y)
    d = rng.standard_normal(y.shape)
    eps = 1e-5
    fd = (W.rhs(m, y + eps * d) - W.rhs(m, y - eps * d)).reshape(-1) / (2 * eps)
    assert np.linalg.norm(J @ d.reshape(-1) - fd) < 1e-7 * np.linalg.norm(fd)
    P = W.rhs_param_derivatives(m, y)
    base = {k: float(getattr(m, k)) for k in W.SWM_PARAMS}
    for i, k in enumerate(W.SWM_PARAMS):
        p = dict(base)
        p[k] += 7.0
        diff = (W.rhs(m, y, p) - W.rhs(m, y, base)).reshape(-1) / 7.0
        # the differences carry the rounding of the whole right-hand side (|F| >> dF/dnu)
        assert np.abs(P[i] - diff).max() <= 1e-5 * np.abs(diff).max()
