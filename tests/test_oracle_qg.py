"""The reference's QG tests (tests/models/test_qg_*.py, tests/core/test_transforms.py)
re-expressed against the oracle, plus operator invariants."""

import numpy as np
import pytest

from oracle import qg

TWO = dict(nx=16, ny=16, H=(500.0, 4500.0), g_prime=(9.81, 0.025))


def test_zero_pv_zero_tendency():  # test_qg_baroclinic.py:79-94
    m = qg.baroclinic_model(**TWO)
    dq = qg.vector_field(m, np.zeros((2, m.grid.Ny, m.grid.Nx)))
    assert np.max(np.abs(dq)) < 1e-12
    mb = qg.barotropic_model(nx=16, ny=16)  # test_qg_barotropic.py:86-95
    assert np.max(np.abs(qg.vector_field(mb, np.zeros((18, 18))))) < 1e-12


def test_wind_top_layer_only():  # test_qg_baroclinic.py:96-112
    m = qg.baroclinic_model(**TWO, wind_amplitude=1e-10)
    dq = qg.vector_field(m, np.zeros((2, 18, 18)))
    assert np.max(np.abs(dq[0])) > 0
    assert np.max(np.abs(dq[1])) < 1e-15


def test_boundary_conditions():  # test_qg_baroclinic.py:166-183
    m = qg.baroclinic_model(**TWO)
    q = qg.apply_boundary_conditions(m, np.ones((2, 18, 18)))
    assert np.all(q[:, 0] == 0) and np.all(q[:, -1] == 0)
    assert np.all(q[:, :, 0] == 0) and np.all(q[:, :, -1] == 0)
    assert np.all(q[:, 1:-1, 1:-1] == 1)


def test_modal_roundtrip():  # test_transforms.py:119-152
    for H, g in (((500.0, 4500.0), (9.81, 0.025)), ((300.0, 700.0, 4000.0), (9.81, 0.025, 0.0125))):
        md = qg.vertical_modes(H, g, 1e-4)
        np.testing.assert_allclose(md.Cl2m @ md.Cm2l, np.eye(len(H)), atol=1e-12)
        x = np.random.default_rng(0).normal(size=(len(H), 5, 5))
        np.testing.assert_allclose(md.to_layer(md.to_modal(x)), x, atol=1e-12)
        assert np.all(md.rossby_radii[np.isfinite(md.rossby_radii)] > 0)
    md = qg.vertical_modes((1000.0,), (9.81,), 1e-4)
    assert md.Cl2m.shape == (1, 1)


def test_reference_eigs_are_sorted_and_differ():
    # transforms.py:194: eigh of the symmetrised A (sorted); not the eigenvalues of A itself
    H, g = (400.0, 1100.0, 2600.0), (9.81, 0.025, 0.0125)
    ref = qg.vertical_modes(H, g, 9.375e-5, eigs="reference").eigenvalues
    con = qg.vertical_modes(H, g, 9.375e-5, eigs="consistent").eigenvalues
    assert np.all(np.diff(ref) >= 0) and np.all(np.diff(con) >= 0)
    np.testing.assert_allclose(con, [2.48e-5, 6.61e-2, 1.74e-1], rtol=5e-3)
    assert ref[0] < 0  # the symmetrised matrix is indefinite: recorded, not fixed


def test_inversion_solves_layer_system():
    # (lap - f0^2 A) psi = q in layer space, with the full-array operator, before ring zeroing
    m = qg.baroclinic_model(nx=20, ny=24, Lx=1e6, Ly=1.2e6)
    g = m.grid
    rng = np.random.default_rng(1)
    q = qg.zero_boundaries(rng.normal(size=(3, g.Ny, g.Nx)) * 1e-6)
    qm = m.modes.to_modal(q)
    pm = qg.helmholtz_dst(qm, g.dx, g.dy, m.helmholtz_lambdas)
    r = qm - qg.helmholtz_apply_full(pm, g.dx, g.dy, m.helmholtz_lambdas)
    assert np.linalg.norm(r) / np.linalg.norm(qm) < 1e-12


def test_dst1_matrix_orthonormal():
    for n in (5, 17, 66):
        S = qg.dst1_matrix(n)
        np.testing.assert_allclose(S @ S, np.eye(n), atol=1e-12)
        np.testing.assert_allclose(S, S.T, atol=0)


def test_dst_matrix_sandwich_equals_scipy():
    # the GEMM formulation used on the GPU: psi = S_y ((S_y q S_x) / Lambda) S_x
    rng = np.random.default_rng(2)
    ny, nx, dx, dy, lam = 13, 9, 0.3, 0.2, 0.7
    q = rng.normal(size=(ny, nx))
    Sy, Sx = qg.dst1_matrix(ny), qg.dst1_matrix(nx)
    L = qg.dst1_eigenvalues(ny, dy)[:, None] + qg.dst1_eigenvalues(nx, dx)[None, :] - lam
    psi = Sy @ ((Sy @ q @ Sx) / L) @ Sx
    np.testing.assert_allclose(psi, qg.helmholtz_dst(q, dx, dy, lam), atol=1e-12)


def test_arakawa_invariants():
    # Arakawa (1966) in a closed basin: psi = 0 on the ring gives sum psi J = 0 (energy) for
    # any q; q = 0 on the ring as well gives sum q J = 0 (enstrophy).
    rng = np.random.default_rng(3)
    psi = qg.zero_boundaries(rng.normal(size=(20, 23)))
    q = rng.normal(size=(20, 23))
    for qq, enstrophy in ((q, False), (qg.zero_boundaries(q), True)):
        Jf = np.zeros_like(psi)
        Jf[1:-1, 1:-1] = qg.arakawa_jacobian(psi, qq, 0.7, 1.3)
        scale = np.sum(np.abs(Jf))
        assert abs(np.sum(psi * Jf)) < 1e-13 * scale
        if enstrophy:
            assert abs(np.sum(qq * Jf)) < 1e-13 * scale


def test_arakawa_on_polynomials():
    # J(x, y) = 1 and J(y, x) = -1 exactly for linear fields
    g = qg.Grid(8, 6, 8.0, 3.0)
    x = np.arange(g.Nx) * g.dx
    y = np.arange(g.Ny) * g.dy
    X, Y = np.meshgrid(x, y)
    np.testing.assert_allclose(qg.arakawa_jacobian(X, Y, g.dx, g.dy), 1.0, atol=1e-12)
    np.testing.assert_allclose(qg.arakawa_jacobian(Y, X, g.dx, g.dy), -1.0, atol=1e-12)


@pytest.mark.parametrize("scheme", ["heun", "ssprk3", "tsit5"])
def test_integrate_finite_and_wind_develops_flow(scheme):  # test_qg_baroclinic.py:185-223
    m = qg.baroclinic_model(**TWO, lateral_viscosity=50.0, wind_amplitude=1e-10)
    q = qg.integrate(m, np.zeros((2, 18, 18)), 100.0, 36, scheme)
    assert np.all(np.isfinite(q))
    assert np.max(np.abs(q[0, 2:-2, 2:-2])) > 1e-10


def test_scheme_order():
    # halving dt reduces the error like dt^p for a smooth linear problem
    m = qg.baroclinic_model(nx=12, ny=12, Lx=1e6, Ly=1e6, lateral_viscosity=2e3, wind_amplitude=1e-10)
    rng = np.random.default_rng(4)
    q0 = qg.zero_boundaries(rng.normal(size=(3, 14, 14)) * 1e-7)
    T = 8 * 3600.0
    ref = qg.integrate(m, q0, T / 256, 256, "tsit5")
    for scheme, p in (("heun", 2), ("ssprk3", 3)):
        e1 = np.linalg.norm((qg.integrate(m, q0, T / 8, 8, scheme) - ref)[:, 1:-1, 1:-1])
        e2 = np.linalg.norm((qg.integrate(m, q0, T / 16, 16, scheme) - ref)[:, 1:-1, 1:-1])
        assert np.log2(e1 / e2) > p - 0.3


def test_diagnose():  # test_qg_baroclinic.py:225-259
    m = qg.baroclinic_model(**TWO)
    d = qg.diagnose(m, 0.01 * np.ones((2, 18, 18)))
    assert d["kinetic_energy"].shape == (2,) and np.all(d["kinetic_energy"] >= 0)
    assert np.isfinite(d["total_enstrophy"])


def test_float32_close_to_float64():
    m = qg.baroclinic_model(nx=30, ny=30, Lx=5.12e6, Ly=5.12e6, lateral_viscosity=100.0,
                            bottom_drag=1e-7, wind_amplitude=9.8e-11)
    rng = np.random.default_rng(5)
    q = qg.zero_boundaries(rng.normal(size=(3, 32, 32)) * 1e-6)
    d64 = qg.vector_field(m, q)
    d32 = qg.vector_field(m, q.astype(np.float32))
    assert d32.dtype == np.float32
    assert np.linalg.norm(d32 - d64) / np.linalg.norm(d64) < 1e-5
