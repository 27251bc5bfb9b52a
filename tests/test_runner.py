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


@pytest.mark.gpu
def test_state_stats_kernel_matches_host_reduction():
    """qg_state_stats (min / mean / max over the finite entries, non-finite count) against the
    same reduction in float64 on the host, with NaN and inf entries planted in the field."""
    m, _, q0 = _model()
    plan = m.plan()
    q = torch.tensor(q0, dtype=torch.float32, device="cuda").reshape(-1)
    q[5] = float("nan")
    q[77] = float("inf")
    q[-1] = float("-inf")
    got = plan.state_stats(q).cpu().numpy()
    h = q.cpu().double().numpy()
    f = h[np.isfinite(h)]
    assert got[0] == f.min() and got[2] == f.max() and got[3] == 3
    assert abs(got[1] - f.mean()) <= 1e-12 * np.abs(f).max()
    allbad = torch.full_like(q, float("nan"))
    got = plan.state_stats(allbad).cpu().numpy()
    assert np.isnan(got[:3]).all() and got[3] == q.numel()


@pytest.mark.gpu
def test_runner_writes_snapshots_and_restart(tmp_path):
    """With output_dir the runner writes snapshots.zarr (the saved states, appended while the
    run goes on) and final_state.zarr; restarting from final_state.zarr and running the second
    half gives the bits of one run over both halves (``_run.py:346-364,840-862``)."""
    from somax_gb300 import io as qio

    m, _, q0 = _model()
    dt = 1200.0
    ts = [0.0, 4 * dt, 8 * dt]
    s0 = sg.BaroclinicQGState(q=torch.tensor(q0, dtype=torch.float32, device="cuda"))
    res = runner.chunked_integrate_with_diagnostics(m, s0, ts, dt, solver="ssprk3", log=lambda s: None,
                                                    output_dir=tmp_path / "run", attrs={"experiment": "t"})
    snaps = qio.load_dataset(res.snapshots_path)
    assert snaps["q"].dims == ("time", "layer", "y", "x")
    np.testing.assert_array_equal(snaps["time"].values, ts)
    np.testing.assert_array_equal(snaps["q"].values, res.ys.q.cpu().numpy())
    assert snaps.attrs["experiment"] == "t" and snaps.attrs["state_class"] == "BaroclinicQGState"
    final = runner.restart_state(res.final_state_path, m, device="cuda")
    assert torch.equal(final.q, res.ys.q[-1])
    # the first half, then a restart from its final_state.zarr
    half = runner.chunked_integrate_with_diagnostics(m, s0, ts[:2], dt, solver="ssprk3", log=lambda s: None,
                                                     output_dir=tmp_path / "half")
    r0 = runner.restart_state(half.final_state_path, m, device="cuda")
    rest = runner.chunked_integrate_with_diagnostics(m, r0, ts[1:], dt, solver="ssprk3", log=lambda s: None)
    assert torch.equal(rest.ys.q[-1], res.ys.q[-1])
    with pytest.raises(ValueError):
        runner.restart_state(res.final_state_path, sg.BaroclinicQG.create(nx=20, ny=20))
