"""Host-side set-up code of the package against the oracle (no GPU)."""

import numpy as np
import pytest

from oracle import qg as O
from somax_gb300 import tableaus, testcases
from somax_gb300.transforms import ModalTransform, StratificationProfile, coupling_matrix


@pytest.mark.parametrize("H,g", [((500.0, 4500.0), (9.81, 0.025)),
                                 ((400.0, 1100.0, 2600.0), (9.81, 0.025, 0.0125)),
                                 (testcases.H5, testcases.G5), ((4000.0,), (0.0055,))])
def test_modal_transform_matches_oracle(H, g):
    np.testing.assert_allclose(coupling_matrix(H, g), O.coupling_matrix(H, g), rtol=1e-15)
    for eigs in ("consistent", "reference"):
        a = ModalTransform.from_physics(H, g, 9.375e-5, eigs)
        b = O.vertical_modes(H, g, 9.375e-5, eigs)
        np.testing.assert_allclose(a.eigenvalues, b.eigenvalues, rtol=1e-12)
        # the inversion operator Cm2l diag(x) Cl2m is scaling-invariant
        x = np.arange(1, len(H) + 1.0)
        np.testing.assert_allclose(a.Cm2l @ np.diag(x) @ a.Cl2m, b.Cm2l @ np.diag(x) @ b.Cl2m, rtol=1e-10,
                                   atol=1e-12)


def test_stratification_factories():  # test_transforms.py:17-91
    s = StratificationProfile.from_N2_constant(N2=1e-5, depth=4000.0, n_layers=4)
    assert s.nl == 4 and np.allclose(s.H, 1000.0) and s.total_depth == 4000.0
    assert np.isclose(s.g_prime[0], 9.81) and np.allclose(s.g_prime[1:], 1e-5 * 1000.0)
    assert np.all(np.diff(s.rho) > 0)
    e = StratificationProfile.from_N2_exponential(N2_surface=1e-4, scale_depth=500.0, depth=4000.0, n_layers=4)
    assert np.all(np.diff(e.g_prime[1:]) < 0)
    with pytest.raises(ValueError):
        StratificationProfile.from_layers(H=[1.0, 2.0], g_prime=[1.0])


def test_tableaus_consistent():
    for s in ("euler", "heun", "ssprk3", "tsit5"):
        a, b = tableaus.rk_tableau(s)
        assert abs(sum(b) - 1.0) < 1e-12
        assert len(a) == len(b)


def _order_conditions(a, b):
    """Residuals of the Butcher order conditions up to order 4 (c_i = sum_j a_ij)."""
    n = len(b)
    A = np.zeros((n, n))
    for i, row in enumerate(a):
        A[i, :len(row)] = row
    b = np.asarray(b, dtype=float)
    c = A.sum(axis=1)
    return [b.sum() - 1, b @ c - 1 / 2,
            b @ c**2 - 1 / 3, b @ A @ c - 1 / 6,
            b @ c**3 - 1 / 4, (b * c) @ A @ c - 1 / 8, b @ A @ c**2 - 1 / 12, b @ A @ A @ c - 1 / 24]


def test_tableau_orders():
    """Each scheme meets the order conditions of its order (Euler 1, Heun 2, SSP-RK3 3, Tsit5 at
    least 4 to the rounding of its published coefficients), and Tsit5's stage times are the
    published c = 0.161, 0.327, 0.9, 0.98002554..., 1, 1."""
    n_cond = {"euler": 1, "heun": 2, "ssprk3": 4, "tsit5": 8}
    for s, k in n_cond.items():
        a, b = tableaus.rk_tableau(s)
        r = _order_conditions(a, b)[:k]
        assert max(abs(x) for x in r) < 1e-12, (s, r)
    a, _ = tableaus.rk_tableau("tsit5")
    c = [sum(row) for row in a]
    np.testing.assert_allclose(c, [0.0, 0.161, 0.327, 0.9, 0.9800255409045097, 1.0], rtol=0, atol=1e-13)


def test_tableau_copies_agree():
    """The library's Tsit5 tableau (somax_gb300/csrc/qg_plan.cu) and the float64 oracle's are the
    host tableau, digit for digit."""
    import re
    from pathlib import Path

    from oracle import qg as OQ

    a, b = tableaus.rk_tableau("tsit5")
    src = (Path(__file__).resolve().parents[1] / "somax_gb300" / "csrc" / "qg_plan.cu").read_text()
    block = src[src.index("static const Tableau tsit5"):]
    block = block[:block.index("};")]
    nums = [float(x) for x in re.findall(r"-?\d+\.\d+(?:e-?\d+)?|(?<![\w.])-?\d+(?![\w.])", block.split("=", 1)[1])]
    n = nums[0]
    assert n == 6
    A = np.array(nums[1:37]).reshape(6, 6)
    B = np.array(nums[37:43])
    for i, row in enumerate(a):
        np.testing.assert_array_equal(A[i, :len(row)], row)
        assert np.all(A[i, len(row):] == 0)
    np.testing.assert_array_equal(B, b)
    for i, row in enumerate(a):
        np.testing.assert_array_equal(OQ._TSIT5_A[i], row)
    np.testing.assert_array_equal(OQ._TSIT5_B[:6], b)


def test_initial_pv_properties():
    cfg = testcases.C1
    q = testcases.initial_pv(cfg, seed=3)
    assert q.shape == (1, 66, 66)
    assert np.all(q[:, 0] == 0) and np.all(q[:, :, -1] == 0)
    # relative vorticity of the inverted field has the requested RMS
    m = O.baroclinic_model(nx=64, ny=64, Lx=cfg.L, Ly=cfg.L, H=cfg.H, g_prime=cfg.g_prime)
    psi = O.invert_pv(m, q)
    zeta = O.laplacian(psi, m.grid.dx, m.grid.dy)[0, 1:-1, 1:-1]
    assert 0.8e-6 < np.sqrt(np.mean(zeta**2)) < 1.2e-6
    q2 = testcases.initial_pv(testcases.C2, seed=3)
    assert q2.shape == (3, 130, 130)
    r = np.sqrt(np.mean(q2[:, 1:-1, 1:-1] ** 2, axis=(1, 2)))
    np.testing.assert_allclose(r / r[0], [1.0, 400 / 1100, 400 / 2600], rtol=1e-12)
    assert np.array_equal(testcases.initial_pv(testcases.C2, seed=3), q2)


def test_wind_amplitude_convention():
    # gfd_testcases.py:250-251: tau0 = 0.08 Pa scaled by 2 pi / (Ly rho0) -> 1.3e-10 at Ly = 4000 km
    assert abs(testcases.wind_amplitude(0.08, 4e6) - 1.2566e-10) < 1e-14
    assert abs(testcases.wind_amplitude(0.08) - 9.817e-11) < 1e-14


def test_deformation_radius_config1():
    cfg = testcases.C1
    lam = testcases.F0**2 / (cfg.g_prime[0] * cfg.H[0])
    assert abs(1 / np.sqrt(lam) - 5.0e4) < 1e-6
