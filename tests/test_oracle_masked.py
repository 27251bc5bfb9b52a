"""The masked-basin oracle (CPU): the capacitance-matrix correction of the DST-I solve equals
a direct sparse solve of the same discrete problem, psi vanishes on the land boundary, and
with no land the masked model is the unmasked one."""

import numpy as np
import pytest

from oracle import masked as OM
from oracle import qg as O
from somax_gb300 import testcases as tc


def test_land_mask_shape_fraction_and_ring():
    m = tc.land_mask(60, 50, frac=0.15, seed=3)
    assert m.shape == (62, 52) and m.dtype == np.uint8
    assert np.all(m[0] == 0) and np.all(m[-1] == 0) and np.all(m[:, 0] == 0) and np.all(m[:, -1] == 0)
    assert abs((m[1:-1, 1:-1] == 0).mean() - 0.15) < 0.01
    assert np.array_equal(m, tc.land_mask(60, 50, frac=0.15, seed=3))


@pytest.mark.parametrize("lam", [0.0, 2.5e-11])
def test_capacitance_equals_direct_solve(lam):
    ny, nx = 26, 30
    mask = tc.land_mask(ny, nx, frac=0.2, seed=1)
    dx, dy = 1e5, 1.2e5
    rhs = np.random.default_rng(2).standard_normal((ny + 2, nx + 2)) * 1e-6
    rhs = np.where(OM.land(mask), 0.0, rhs)
    a = OM.helmholtz_capacitance(rhs, dx, dy, lam, mask)
    b = OM.helmholtz_masked(rhs, dx, dy, lam, mask)
    assert np.linalg.norm(a - b) <= 1e-10 * np.linalg.norm(b)
    B = OM.boundary_points(mask)
    assert len(B) > 0 and np.abs(b.reshape(-1)[B]).max() == 0.0
    assert OM.helmholtz_residual(b, rhs, dx, dy, lam, mask) < 1e-12


def test_no_land_is_the_unmasked_model():
    m = O.baroclinic_model(nx=20, ny=16, Lx=1e6, Ly=8e5, lateral_viscosity=50.0, bottom_drag=1e-7,
                           wind_amplitude=1e-10, biharmonic_viscosity=1e9)
    q = np.random.default_rng(4).standard_normal((3, 18, 22)) * 1e-6
    mask = np.ones((18, 22), np.uint8)
    mask[0] = mask[-1] = 0
    mask[:, 0] = mask[:, -1] = 0
    assert len(OM.boundary_points(mask)) == 0
    assert np.allclose(OM.invert_pv(m, q, mask), O.invert_pv(m, q), rtol=1e-10, atol=1e-14 * np.abs(q).max() * 1e12)
    a, b = OM.vector_field(m, q, mask), O.vector_field(m, q)
    assert np.linalg.norm(a - b) <= 1e-10 * np.linalg.norm(b)


def test_masked_rhs_is_zero_on_land():
    m = O.baroclinic_model(nx=24, ny=20, Lx=1e6, Ly=8e5, lateral_viscosity=50.0, wind_amplitude=1e-10)
    mask = tc.land_mask(20, 24, frac=0.15, seed=5)
    q = np.random.default_rng(6).standard_normal((3, 22, 26)) * 1e-6
    dq = OM.vector_field(m, q, mask)
    assert np.all(dq[:, OM.land(mask)] == 0)
    psi = OM.invert_pv(m, q, mask)
    assert np.all(psi[:, OM.land(mask)] == 0)
