"""The chunked runner (``somax_gb300/runner.py``, mirroring ``cli/_run.py:504-700``): its diagnostic
grid on CPU; on the GPU, chunked integration equals one integrate call per chunk, the snapshots
land on the save times, and a non-finite state aborts with IntegrationDivergedError."""

import numpy as np
import pytest
import torch

import somax_gb300 as sg
from oracle import qg as O
from somax_gb300 import runner
from somax_gb300 import testcases as tc


def test_diagnostic_grid():
    ts = np.array([0.0, 10.0, 30.0])
    g, idx = runner.build_diagnostic_grid(ts, 1)
    assert np.array_equal(g, ts) and idx == {0, 1, 2}
    g, idx = runner.build_diagnostic_grid(ts, 4)
    assert np.allclose(g, [0, 2.5, 5, 7.5, 10, 15, 20, 25, 30])
    assert idx == {0, 4, 8} and np.array_equal(g[sorted(idx)], ts)


def _model():
    cfg = tc.C2
    kw = dict(cfg.model_kwargs(), nx=40, ny=40, Lx=1.6e6, Ly=1.6e6)
    m = sg.BaroclinicQG.create(**kw, precision="bf16x3")
    o = O.baroclinic_model(nx=40, ny=40, Lx=1.6e6, Ly=1.6e6, f0=kw["f0"], beta=kw["beta"], H=cfg.H,
                           g_prime=cfg.g_prime, bottom_drag=cfg.bottom_drag, wind_amplitude=kw["wind_amplitude"],
                           biharmonic_viscosity=cfg.biharmonic_viscosity)
    q0 = tc.kminus3_field(40, 3, 3) * 1e-6
    return m, o, q0


@pytest.mark.gpu
def test_chunked_integration_matches_per_chunk_integrate():
    m, o, q0 = _model()
    dt, save_ts = 1200.0, [0.0, 6 * 1200.0, 12 * 1200.0]
    lines = []
    res = runner.chunked_integrate_with_diagnostics(
        m, sg.BaroclinicQGState(q=torch.tensor(q0, dtype=torch.float32, device="cuda")), save_ts, dt,
        diagnostics_per_save=3, solver="ssprk3", log=lines.append)
    assert res.ys.q.shape == (3, 3, 42, 42) and len(res.diagnostics) == 6 and len(lines) == 7
    # the runner re-applies the BC at every chunk (each chunk is an integrate call), as the
    # reference's does; the oracle chains the same chunks
    y = q0
    for _ in range(6):
        y = O.integrate(o, y, dt, 2, "ssprk3")
    got = res.ys.q[-1].cpu().double().numpy()
    assert np.linalg.norm(got - y) / np.linalg.norm(y) < 1e-5
    assert all(np.isfinite(r["total_kinetic_energy"]) for r in res.diagnostics)


@pytest.mark.gpu
def test_non_finite_state_aborts():
    m, _, q0 = _model()
    q = torch.tensor(q0, dtype=torch.float32, device="cuda")
    q[1, 10, 10] = float("nan")  # planted on the host side of the call
    with pytest.raises(runner.IntegrationDivergedError):
        runner.chunked_integrate_with_diagnostics(m, sg.BaroclinicQGState(q=q), [0.0, 2400.0, 4800.0], 1200.0,
                                                  solver="ssprk3", log=lambda s: None)
