"""The chunked runner (``somax_gb300/runner.py``, mirroring ``cli/_run.py:504-700``): its diagnostic
grid and diagnostics flattening on CPU; on the GPU, chunked integration equals one integrate
call per chunk, the snapshots land on the save times, a restart continues the run bit for bit,
and a non-finite state aborts with IntegrationDivergedError, for the QG model and for the
shallow-water and reparameterised models (state h, u, v)."""

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


def test_flatten_diagnostics():
    """``_flatten_diagnostics``: 0-d fields as floats, per-layer vectors as <field>_layer_<i>,
    fields left out; the headline line in the reference's priority order."""
    import dataclasses

    @dataclasses.dataclass
    class D:
        total_energy: torch.Tensor
        energy: torch.Tensor
        field: torch.Tensor
        radii: np.ndarray
        none: object = None

    d = D(torch.tensor(3.0), torch.tensor([1.0, 2.0]), torch.zeros(4, 5), np.array([7.0]))
    flat = runner.flatten_diagnostics(d)
    assert flat == {"total_energy": 3.0, "energy_layer_0": 1.0, "energy_layer_1": 2.0, "radii_layer_0": 7.0}

    class M:
        def diagnose(self, s):
            return d

    line, f2 = runner.physical_scalars(M(), None)
    assert line == "total_energy=3.000000e+00" and f2 == flat

    class Bad:
        def diagnose(self, s):
            raise ValueError("x")

    assert runner.physical_scalars(Bad(), None) == ("diagnose failed: ValueError: x", {})


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


@pytest.mark.gpu
def test_runner_shallow_water_jet(tmp_path):
    """The reference's swm_jet test case (16^2 here) through the runner: statistics of h, u and
    v, the total energy in every record, chunks equal to one integrate call each, snapshots of
    the three fields, and a restart from final_state.zarr that continues the run bit for bit."""
    from somax_gb300 import io as qio

    m, s0 = sg.baroclinic_instability_swm(nx=16, ny=16, lateral_viscosity=1000.0)
    dt, ts = 20.0, [0.0, 600.0, 1200.0]
    lines = []
    res = runner.chunked_integrate_with_diagnostics(m, s0, ts, dt, diagnostics_per_save=2, log=lines.append,
                                                    output_dir=tmp_path / "run", attrs={"experiment": "jet"})
    assert len(lines) == 5 and "total_energy=" in lines[-1]
    assert set(res.diagnostics[0]["stats"]) == {"h", "u", "v"}
    assert all(np.isfinite(r["total_energy"]) for r in res.diagnostics)
    assert res.ys.h.shape == (3, 2, 18, 18)
    s = s0
    for t0 in (0.0, 300.0, 600.0, 900.0):
        sol = m.integrate(s, t0, t0 + 300.0, dt)
        s = sg.MultilayerSW2DState(sol.ys.h[-1], sol.ys.u[-1], sol.ys.v[-1])
    assert torch.equal(s.u, res.ys.u[-1]) and torch.equal(s.h, res.ys.h[-1])
    snaps = qio.load_dataset(res.snapshots_path)
    assert snaps["v"].dims == ("time", "layer", "y", "x") and snaps.attrs["state_class"] == "MultilayerSW2DState"
    np.testing.assert_array_equal(snaps["v"].values, res.ys.v.cpu().numpy())
    half = runner.chunked_integrate_with_diagnostics(m, s0, ts[:2], dt, log=lambda s: None,
                                                     output_dir=tmp_path / "half")
    r0 = runner.restart_state(half.final_state_path, m, device="cuda")
    rest = runner.chunked_integrate_with_diagnostics(m, r0, ts[1:], dt, log=lambda s: None)
    whole = runner.chunked_integrate_with_diagnostics(m, s0, ts, dt, log=lambda s: None)  # the same chunks
    assert torch.equal(rest.ys.h[-1], whole.ys.h[-1]) and torch.equal(rest.ys.v[-1], whole.ys.v[-1])
    bad = sg.MultilayerSW2DState(s0.h.clone(), s0.u.clone(), s0.v.clone())
    bad.h[0, 8, 8] = float("nan")
    with pytest.raises(runner.IntegrationDivergedError):
        runner.chunked_integrate_with_diagnostics(m, bad, ts, dt, log=lambda s: None)


@pytest.mark.gpu
def test_runner_reparameterized_double_gyre():
    m, s0 = sg.doublegyre_reparameterized_qg(nx=16, ny=16)
    res = runner.chunked_integrate_with_diagnostics(m, s0, [0.0, 500.0, 1000.0], 10.0, log=lambda s: None)
    assert set(res.diagnostics[-1]["stats"]) == {"h", "u", "v"}
    assert all(r["stats"][k]["nan"] == 0 for r in res.diagnostics for k in "huv")
    assert np.isfinite(res.diagnostics[-1]["total_energy"])
