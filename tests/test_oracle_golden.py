"""Pin the oracle against the reference's own printed known answers (tests/golden).

These are the only exact numbers somax publishes for the operators on the QG path:
DST-I Poisson/Helmholtz (step10/step11 tutorials) and the 5-point Laplacian + Tsit5
stepping + its gradient (step07 tutorial).
"""

import json
import pathlib

import numpy as np
import pytest

from oracle import qg

GOLD = json.loads((pathlib.Path(__file__).parent / "golden" / "tutorial_values.json").read_text())


def _unit_grid(n):
    g = qg.Grid(n, n, 1.0, 1.0)
    x = np.arange(g.Nx) * g.dx
    X, Y = np.meshgrid(x, x)
    return g, X, Y


def test_poisson_dirichlet_64():
    # step10 cell 4: sin(pi x) sin(pi y) manufactured solution, L2 error over the interior
    g, X, Y = _unit_grid(64)
    rhs = -2 * np.pi**2 * np.sin(np.pi * X) * np.sin(np.pi * Y)
    exact = np.sin(np.pi * X) * np.sin(np.pi * Y)
    phi = qg.helmholtz_dst(rhs, g.dx, g.dy, 0.0)
    err = np.sqrt(np.mean((phi[1:-1, 1:-1] - exact[1:-1, 1:-1]) ** 2))
    # printed by the reference in float32: agreement to 1e-6 relative
    assert err == pytest.approx(GOLD["poisson_dirichlet_64_l2"]["value"], rel=1e-6)


def test_poisson_dirichlet_convergence():
    d = GOLD["poisson_dirichlet_convergence"]
    for n, ref in zip(d["n"], d["l2"]):
        g, X, Y = _unit_grid(n)
        rhs = -2 * np.pi**2 * np.sin(np.pi * X) * np.sin(np.pi * Y)
        exact = np.sin(np.pi * X) * np.sin(np.pi * Y)
        phi = qg.helmholtz_dst(rhs, g.dx, g.dy, 0.0)
        err = np.sqrt(np.mean((phi[1:-1, 1:-1] - exact[1:-1, 1:-1]) ** 2))
        assert float(f"{err:.2e}") == ref  # printed with 3 significant digits


def test_helmholtz_amplitudes():
    d = GOLD["helmholtz_max_abs"]
    g, X, Y = _unit_grid(64)
    rhs = np.sin(np.pi * X) * np.sin(np.pi * Y)
    for lam, ref in zip(d["lambda"], d["max_abs_phi"]):
        amp = np.max(np.abs(qg.helmholtz_dst(rhs, g.dx, g.dy, lam)[1:-1, 1:-1]))
        assert float(f"{amp:.6f}") == ref


def test_helmholtz_lambda0_is_poisson():
    g, X, Y = _unit_grid(64)
    rhs = np.sin(np.pi * X) * np.sin(np.pi * Y)
    d = np.max(np.abs(qg.helmholtz_dst(rhs, g.dx, g.dy, 0.0) - qg.helmholtz_dst(rhs, g.dx, g.dy)))
    assert d == GOLD["helmholtz_lambda0_vs_poisson"]["max_abs_diff"]


def _diffusion_run(nu, n_steps):
    # step07: Diffusion2D(nx=64, Lx=4, nu=0.05), Gaussian sigma 0.3 at (2, 2), periodic BC
    # (diffusion.py:67-69), Tsit5 (core/model.py:75) at dt = 0.002.
    g = qg.Grid(64, 64, 4.0, 4.0)
    x = np.arange(g.Nx) * g.dx
    X, Y = np.meshgrid(x, x)
    u0 = np.exp(-0.5 * (((X - 2.0) / 0.3) ** 2 + ((Y - 2.0) / 0.3) ** 2))

    def f(u):
        return nu * qg.laplacian(qg.enforce_periodic(u), g.dx, g.dy)

    ys = [qg.enforce_periodic(u0)]
    for _ in range(n_steps):
        ys.append(qg.rk_step(f, ys[-1], 0.002, "tsit5"))
    return g, X, Y, ys


def test_diffusion_energy_and_error():
    g, X, Y, ys = _diffusion_run(0.05, 499)  # ts = arange(0, 1, 0.002): last save at 0.998
    E = [0.5 * np.sum(y[1:-1, 1:-1] ** 2) * g.dx * g.dy for y in (ys[0], ys[-1])]
    d = GOLD["diffusion_energy"]
    assert float(f"{E[0]:.6f}") == d["initial"]
    assert float(f"{E[1]:.6f}") == d["final"]
    assert float(f"{E[1] / E[0]:.4f}") == d["ratio"]
    st = np.sqrt(0.3**2 + 2 * 0.05 * 0.998)
    ua = (0.3**2 / st**2) * np.exp(-0.5 * (((X - 2) / st) ** 2 + ((Y - 2) / st) ** 2))
    err = np.max(np.abs(ys[-1] - ua)[1:-1, 1:-1])
    assert float(f"{err:.6f}") == GOLD["diffusion_max_abs_error"]["value"]


def test_diffusion_gradient():
    # step07 cell 18: d/dnu sum(u(t=0.5)^2), 250 Tsit5 steps; central FD in float64
    h = 1e-6

    def L(nu):
        return np.sum(_diffusion_run(nu, 250)[3][-1] ** 2)

    dL = (L(0.05 + h) - L(0.05 - h)) / (2 * h)
    assert dL == pytest.approx(GOLD["diffusion_dL_dnu"]["value"], rel=1e-6)
