"""The float64 derivative oracle and the host side of the adjoint (CPU).

* ``oracle.adjoint``'s central differences are exact for the quadratic RHS: two different
  steps give the same directional derivative to rounding.
* ``somax_gb300.adjoint``'s checkpointed RK adjoint (the host logic around ``qg_rhs_vjp``)
  against torch autograd through an explicit Butcher loop, on a CPU stand-in for the plan
  whose RHS is a small quadratic map with the same ring semantics.
"""

import numpy as np
import pytest
import torch

from oracle import adjoint as OA
from oracle import qg as O
from somax_gb300 import adjoint as A
from somax_gb300.tableaus import rk_tableau


def _q(shape, seed, scale=1e-6):
    return scale * np.random.default_rng(seed).standard_normal(shape)


@pytest.mark.parametrize("baro", [False, True])
def test_oracle_central_difference_is_exact_for_the_quadratic_rhs(baro):
    if baro:
        m = O.barotropic_model(nx=9, ny=7, lateral_viscosity=50.0, bottom_drag=1e-7, wind_amplitude=1e-10,
                               biharmonic_viscosity=1e9)
        shape = (9, 11)
    else:
        m = O.baroclinic_model(nx=8, ny=6, Lx=1e6, Ly=8e5, lateral_viscosity=50.0, bottom_drag=1e-7,
                               wind_amplitude=1e-10, biharmonic_viscosity=1e9)
        shape = (3, 8, 10)
    q, d = _q(shape, 1), _q(shape, 2)
    a = OA.rhs_directional(m, q, d)
    h = 1e-3
    b = (OA.rhs(m, q + h * d) - OA.rhs(m, q - h * d)) / (2 * h)
    assert np.linalg.norm(a - b) <= 1e-9 * np.linalg.norm(a)
    # the dense Jacobian reproduces the directional derivative
    Jm = OA.rhs_jacobian(m, q)
    assert np.linalg.norm(Jm @ d.reshape(-1) - a.reshape(-1)) <= 1e-9 * np.linalg.norm(a)
    # parameter derivatives: rhs is affine in each parameter, two step sizes agree
    G = OA.rhs_param_derivatives(m, q)
    G7 = OA.rhs_param_derivatives(m, q, scale=7.0)
    for k in range(4):
        assert np.linalg.norm(G[k] - G7[k]) <= 1e-9 * max(np.linalg.norm(G[k]), 1e-300)


def test_oracle_invert_vjp_is_the_transpose():
    m = O.baroclinic_model(nx=7, ny=5, Lx=1e6, Ly=8e5)
    shape = (3, 7, 9)
    q, pb = _q(shape, 3), np.random.default_rng(4).standard_normal(shape)
    lhs = float(np.sum(OA.invert_vjp(m, pb) * q))
    rhs = float(np.sum(pb * O.invert_pv(m, q)))
    assert lhs == pytest.approx(rhs, rel=1e-10)


# ------------------------------------------------------------------------------------------
# host logic of the checkpointed adjoint, on a CPU stand-in plan
# ------------------------------------------------------------------------------------------
def _ring_zero(y):
    y = y.clone()
    y[..., 0, :] = 0
    y[..., -1, :] = 0
    y[..., :, 0] = 0
    y[..., :, -1] = 0
    return y


def _fake_rhs(y, p, apply_bc):
    """A quadratic map with the QG RHS's structure: interior terms from the BC'd input,
    a parameter-scaled constant forcing everywhere (the wind), linear damping terms."""
    yb = _ring_zero(y) if apply_bc else y
    lap = torch.zeros_like(yb)
    lap[..., 1:-1, 1:-1] = (yb[..., 2:, 1:-1] + yb[..., :-2, 1:-1] + yb[..., 1:-1, 2:] + yb[..., 1:-1, :-2]
                            - 4 * yb[..., 1:-1, 1:-1])
    adv = torch.zeros_like(yb)
    adv[..., 1:-1, 1:-1] = yb[..., 1:-1, 1:-1] * (yb[..., 1:-1, 2:] - yb[..., 1:-1, :-2])
    n = yb.shape[-1]
    forcing = torch.sin(torch.linspace(0, 3, n, dtype=yb.dtype)).expand_as(yb)
    return -adv + p[0] * lap - p[1] * yb + p[2] * forcing


class FakePlan:
    def rhs(self, q, p, apply_bc=False, out=None):
        return _fake_rhs(q, p, apply_bc).contiguous()

    def rhs_vjp(self, q, p, g, apply_bc=False, want_params=True):
        with torch.enable_grad():  # backward passes run with grad mode off
            qq = q.detach().clone().requires_grad_(True)
            pp = p.detach().clone().requires_grad_(True)
            out = _fake_rhs(qq, pp, apply_bc)
            gq, gp = torch.autograd.grad(out, (qq, pp), g)
        return gq, (gp if want_params else None)

    def step_vjp(self, y0, p, dt, scheme, g):
        # the library's qg_step_vjp runs this algebra in one call; here its torch form
        return A.step_vjp_torch(self, y0, p, dt, scheme, g)

    def step(self, q, p, dt, n, scheme, apply_bc=True):
        a, b = rk_tableau(scheme)
        y = _ring_zero(q) if apply_bc else q.clone()
        for _ in range(n):
            ks = []
            for s in range(len(b)):
                ys = y + dt * sum(aij * ks[j] for j, aij in enumerate(a[s])) if s else y
                ks.append(self.rhs(ys, p, True))
            y = y + dt * sum(bj * k for bj, k in zip(b, ks))
        q.copy_(y)
        return q


def _reference_loop(q0, p, dt, n, scheme, apply_bc):
    a, b = rk_tableau(scheme)
    y = _ring_zero(q0) if apply_bc else q0
    for _ in range(n):
        ks = []
        for s in range(len(b)):
            ys = y + dt * sum(aij * ks[j] for j, aij in enumerate(a[s])) if s else y
            ks.append(_fake_rhs(ys, p, True))
        y = y + dt * sum(bj * k for bj, k in zip(b, ks))
    return y


@pytest.mark.parametrize("scheme", ["euler", "heun", "ssprk3", "tsit5"])
@pytest.mark.parametrize("n,every", [(7, 3), (6, 10), (5, 1), (0, 4)])
def test_checkpointed_adjoint_matches_autograd(scheme, n, every):
    g = torch.Generator().manual_seed(5)
    q0 = 0.1 * torch.randn((2, 7, 9), generator=g)
    p = torch.tensor([0.05, 0.2, 0.3, 0.0])
    w = torch.randn((2, 7, 9), generator=g)
    dt = 0.1
    for apply_bc in (True, False):
        qa = q0.clone().requires_grad_(True)
        pa = p.clone().requires_grad_(True)
        out = A.integrate(FakePlan(), qa, pa, dt, n, scheme, apply_bc=apply_bc, checkpoint_every=every)
        (out * w).sum().backward()
        qr = q0.clone().requires_grad_(True)
        pr = p.clone().requires_grad_(True)
        ref = _reference_loop(qr, pr, dt, n, scheme, apply_bc)
        (ref * w).sum().backward()
        assert torch.allclose(out, ref.detach(), rtol=1e-5, atol=1e-6)
        assert torch.allclose(qa.grad, qr.grad, rtol=1e-4, atol=1e-6)
        pr_grad = pr.grad if pr.grad is not None else torch.zeros_like(p)  # n = 0: no dependence
        assert torch.allclose(pa.grad, pr_grad, rtol=1e-4, atol=1e-6)
