"""The multilayer shallow-water model on the GPU (``qg_swm_*`` through ``MultilayerShallowWater2D``)
against the float64 restatement ``oracle.swm`` of ``somax/_src/models/swm/multilayer.py``.

Tolerances: the right-hand side is FP32 (as the reference's default JAX dtype), and its
pressure-gradient and PV-flux terms difference large quantities (g h with h ~ 500 m against a
perturbation of a few metres), so each comparison is bounded by max(floor, 4 x the error of
the same restatement run in float32), the floor 2e-5 for one right-hand side and 1e-5 after
20 steps.  Boundary rules are copies and zeros: bit-equal.
"""

import numpy as np
import pytest
import torch

import somax_gb300 as sg
from oracle import swm as W
from somax_gb300 import _lib

pytestmark = pytest.mark.gpu

CASES = [((16, 16), (500.0, 500.0), (9.81, 0.02)),
         ((37, 21), (400.0, 1100.0, 2600.0), (9.81, 0.025, 0.0125)),
         ((64, 48), (500.0,), (9.81,)),
         ((30, 30), (200.0, 356.0, 632.0, 1125.0, 2000.0), (9.81, 0.03, 0.02, 0.0125, 0.008))]


def pair(n, H, gp, bc, nu=300.0, kappa=1e-5, tau=2e-3, Lx=1.2e6, Ly=0.9e6, engine="auto"):
    kw = dict(nx=n[0], ny=n[1], Lx=Lx, Ly=Ly, f0=1e-4, beta=1.6e-11, H=H, g_prime=gp, lateral_viscosity=nu,
              bottom_drag=kappa, wind_amplitude=tau, bc=bc)
    m = sg.MultilayerShallowWater2D.create(n_layers=len(H), engine=engine, **kw)
    return m, W.create(**kw)


def smooth(rng, shape, scale):
    """Smooth random field: white noise smoothed by a few 5-point averages."""
    a = rng.standard_normal(shape)
    for _ in range(4):
        a[..., 1:-1, 1:-1] = (a[..., 1:-1, 1:-1] * 4 + a[..., 2:, 1:-1] + a[..., :-2, 1:-1] + a[..., 1:-1, 2:] +
                              a[..., 1:-1, :-2]) / 8
    return scale * a / np.abs(a).max()


def state(o, seed):
    rng = np.random.default_rng(seed)
    shp = (o.nl, o.Ny, o.Nx)
    h = o.H[:, None, None] + smooth(rng, shp, 4.0)
    u = smooth(rng, shp, 0.3)
    v = smooth(rng, shp, 0.3)
    return np.stack([h, u, v]).astype(np.float32).astype(np.float64)


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def gpu_state(m, y):
    return sg.MultilayerSW2DState(*(torch.tensor(y[k], dtype=torch.float32, device="cuda") for k in range(3)))


def as_np(st):
    return np.stack([st.h.cpu().double().numpy(), st.u.cpu().double().numpy(), st.v.cpu().double().numpy()])


@pytest.mark.parametrize("bc", ["periodic", "wall"])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_rhs_matches_oracle(case, bc):
    n, H, gp = CASES[case]
    m, o = pair(n, H, gp, bc)
    y = state(o, 10 + case)
    # vector_field on the state as given, and the _rhs form (BC applied as it is read)
    got_vf = as_np(m.vector_field(0.0, gpu_state(m, y)))
    ref_vf = np.stack(W.vector_field(o, y[0], y[1], y[2]))
    f32_vf = np.stack(W.vector_field(o, *(y.astype(np.float32))))
    pl = m.plan()
    yd = torch.tensor(y, dtype=torch.float32, device="cuda").reshape(-1)
    got_rhs = pl.rhs(yd, m._param_vector(yd.device), apply_bc=True).view(y.shape).cpu().double().numpy()
    ref_rhs = W.rhs(o, y)
    f32_rhs = W.rhs(o, y.astype(np.float32))
    assert pl.status() == 0
    for got, ref, f32 in ((got_vf, ref_vf, f32_vf), (got_rhs, ref_rhs, f32_rhs)):
        for k in range(3):
            tol = max(2e-5, 4 * rel(f32[k], ref[k]))
            assert rel(got[k], ref[k]) < tol, (k, rel(got[k], ref[k]), tol)


@pytest.mark.parametrize("bc", ["periodic", "wall"])
def test_apply_bc_bit_equal(bc):
    n, H, gp = CASES[1]
    m, o = pair(n, H, gp, bc)
    y = state(o, 5) + np.random.default_rng(6).standard_normal((3, o.nl, o.Ny, o.Nx)).astype(np.float32)
    got = as_np(m.apply_boundary_conditions(gpu_state(m, y)))
    ref = np.stack(W.apply_boundary_conditions(o, y[0], y[1], y[2]))
    assert np.array_equal(got.astype(np.float32), ref.astype(np.float32))


@pytest.mark.parametrize("engine", ["stages", "cluster"])
@pytest.mark.parametrize("scheme", ["heun", "ssprk3", "tsit5"])
@pytest.mark.parametrize("bc", ["periodic", "wall"])
def test_steps_match_oracle(scheme, bc, engine):
    n, H, gp = CASES[1]
    m, o = pair(n, H, gp, bc, engine=engine)
    assert m.plan().engine(scheme)["engine"] == engine
    y = state(o, 20)
    dt = 0.2 * min(o.dx, o.dy) / np.sqrt(9.81 * sum(H))
    got = as_np(m.step(gpu_state(m, y), dt, 20, scheme))
    ref = W.integrate(o, y, dt, 20, scheme)
    f32 = W.integrate(o, y.astype(np.float32), dt, 20, scheme)
    assert m.status() == 0
    for k in range(3):
        tol = max(1e-5, 4 * rel(f32[k], ref[k]))
        assert rel(got[k], ref[k]) < tol, (k, rel(got[k], ref[k]), tol)


def test_reference_physics_on_gpu():
    """``tests/models/test_swm_multilayer.py`` on the GPU path: rest state has zero tendency,
    the wind drives the top layer only, a height bump couples the layers, a short Tsit5
    integration stays finite and the energy is non-negative."""
    m = sg.MultilayerShallowWater2D.create(nx=16, ny=16, n_layers=2, H=(500.0, 500.0), g_prime=(9.81, 0.02))
    Ny, Nx = m.grid.Ny, m.grid.Nx
    h0 = torch.ones((2, Ny, Nx), device="cuda") * torch.tensor([500.0, 500.0], device="cuda")[:, None, None]
    z = torch.zeros_like(h0)
    rest = sg.MultilayerSW2DState(h=h0, u=z, v=z)
    t = m.vector_field(0.0, m.apply_boundary_conditions(rest))
    assert max(float(x.abs().max()) for x in (t.h, t.u, t.v)) < 1e-10
    mw = sg.MultilayerShallowWater2D.create(nx=16, ny=16, n_layers=2, H=(500.0, 500.0), g_prime=(9.81, 0.02),
                                            wind_amplitude=1e-5)
    t = mw.vector_field(0.0, mw.apply_boundary_conditions(rest))
    assert float(t.u[0].abs().max()) > 0 and float(t.u[-1].abs().max()) < 1e-15
    hb = h0.clone()
    hb[0, Ny // 2, Nx // 2] += 1.0
    bump = sg.MultilayerSW2DState(h=hb, u=z, v=z)
    t = m.vector_field(0.0, m.apply_boundary_conditions(bump))
    assert float(t.u[1].abs().max()) > 0
    mv = sg.MultilayerShallowWater2D.create(nx=16, ny=16, n_layers=2, H=(500.0, 500.0), g_prime=(9.81, 0.02),
                                            lateral_viscosity=100.0)
    sol = mv.integrate(bump, t0=0.0, t1=1000.0, dt=10.0)
    assert torch.isfinite(sol.ys.h).all() and torch.isfinite(sol.ys.u).all()
    assert (mv.diagnose(rest).energy >= 0).all()


def test_integrate_saveat_equals_steps_and_nonfinite_flag():
    n, H, gp = CASES[0]
    m, o = pair(n, H, gp, "wall")
    y = state(o, 30)
    dt = 50.0
    sol = m.integrate(gpu_state(m, y), 0.0, 10 * dt, dt, solver="ssprk3", saveat=sg.SaveAt(ts=[0.0, 4 * dt, 10 * dt]))
    one = m.step(gpu_state(m, y), dt, 10, "ssprk3")
    assert torch.equal(sol.ys.h[-1], one.h) and torch.equal(sol.ys.v[-1], one.v)
    bad = y.copy()
    bad[1, 0, 5, 5] = np.nan
    m.step(gpu_state(m, bad), dt, 1, "heun")
    assert m.status() == _lib.K["QG_ERR_NONFINITE"]
    assert m.status() == 0


@pytest.mark.parametrize("scheme", ["euler", "heun", "ssprk3", "tsit5"])
@pytest.mark.parametrize("bc", ["periodic", "wall"])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_cluster_engine_matches_stages(case, bc, scheme):
    """The cluster engine (every step in one thread-block cluster, halo rows from the
    neighbouring CTAs' shared memory) against one launch per stage: the same arithmetic per
    cell, so within 1e-6 after 13 steps (one call of 8 + 5, then one more call)."""
    n, H, gp = CASES[case]
    ms, o = pair(n, H, gp, bc, engine="stages")
    mc, _ = pair(n, H, gp, bc, engine="cluster")
    y = state(o, 40 + case)
    dt = 0.1 * min(o.dx, o.dy) / np.sqrt(9.81 * sum(H))
    a = ms.step(ms.step(gpu_state(ms, y), dt, 13, scheme), dt, 1, scheme, apply_bc=False)
    b = mc.step(mc.step(gpu_state(mc, y), dt, 13, scheme), dt, 1, scheme, apply_bc=False)
    assert ms.status() == 0 and mc.status() == 0
    for x, z in ((a.h, b.h), (a.u, b.u), (a.v, b.v)):
        r = float((x - z).norm() / max(float(x.norm()), 1e-30))
        assert r < 1e-6, r


@pytest.mark.parametrize("bc", ["periodic", "wall"])
def test_cluster_engine_tiny_grid(bc):
    """A 3 x 5 basin on a 16-CTA cluster leaves most CTAs without rows (they still take part in
    every cluster barrier): the cluster engine against the stage engine."""
    ms, o = pair((3, 5), (500.0, 800.0), (9.81, 0.02), bc, engine="stages")
    mc, _ = pair((3, 5), (500.0, 800.0), (9.81, 0.02), bc, engine="cluster")
    y = state(o, 60)
    dt = 0.05 * min(o.dx, o.dy) / np.sqrt(9.81 * 1300.0)
    a = ms.step(gpu_state(ms, y), dt, 9, "ssprk3")
    b = mc.step(gpu_state(mc, y), dt, 9, "ssprk3")
    assert mc.plan().engine("ssprk3")["cluster_ctas"] >= 2
    for x, z in ((a.h, b.h), (a.u, b.u), (a.v, b.v)):
        assert float((x - z).norm()) <= 1e-6 * max(float(x.norm()), 1e-30)


def test_engine_choice_and_nonfinite_flag():
    """AUTO takes the engine that ran the tuning steps faster; the reference's swm_jet basin
    (2 layers, 64^2) fits a cluster; a 3-layer 512^2 basin does not and steps one launch per
    stage (forcing the cluster engine there is an error); a NaN planted in the state raises
    the non-finite flag through the cluster engine."""
    jet0, s0 = sg.baroclinic_instability_swm(nx=64, ny=64, lateral_viscosity=1000.0)
    eng = jet0.plan().engine("tsit5")
    tm = eng["tuning_ms"]
    assert tm["cluster"] > 0 and tm["stages"] > 0, eng
    assert eng["engine"] == ("cluster" if tm["cluster"] < tm["stages"] else "stages"), eng
    print(f"swm_jet64 engine tuning, 32 Tsit5 steps: {eng}")
    jet = sg.MultilayerShallowWater2D.create(nx=64, ny=64, Lx=1e6, Ly=1e6, f0=1e-4, beta=1.6e-11, n_layers=2,
                                             H=(500.0, 4500.0), g_prime=(9.81, 0.025), lateral_viscosity=1000.0,
                                             bottom_drag=1e-7, engine="cluster")
    assert jet.plan().engine("tsit5")["cluster_ctas"] in (16, 8, 4, 2)
    big = sg.MultilayerShallowWater2D.create(nx=512, ny=512, n_layers=3)
    assert big.plan().engine("tsit5")["engine"] == "stages"
    forced = sg.MultilayerShallowWater2D.create(nx=512, ny=512, n_layers=3, engine="cluster")
    z = torch.zeros((3,) + forced.shape, device="cuda")
    with pytest.raises(RuntimeError):
        forced.step(sg.MultilayerSW2DState(z[0] + 500.0, z[1], z[2]), 1.0, 1, "tsit5")
    bad = sg.MultilayerSW2DState(s0.h.clone(), s0.u.clone(), s0.v.clone())
    bad.u[1, 30, 30] = float("nan")
    jet.step(bad, 20.0, 3, "tsit5")
    assert jet.status() == _lib.K["QG_ERR_NONFINITE"]
    assert jet.status() == 0


def test_field_stats_and_profiling_counters():
    """qg_swm_state_stats against a float64 host reduction with NaN / inf planted, and the
    per-launch profiling counters of qg_swm_step: one k_swm_stage launch per stage on the stage
    engine, one k_swm_cluster launch per call on the cluster engine."""
    n, H, gp = CASES[1]
    m, o = pair(n, H, gp, "wall", engine="stages")
    pl = m.plan()
    x = torch.tensor(state(o, 50)[1], dtype=torch.float32, device="cuda").reshape(-1)
    x[3] = float("nan")
    x[40] = float("inf")
    got = pl.field_stats(x).cpu().numpy()
    h = x.cpu().double().numpy()
    f = h[np.isfinite(h)]
    assert got[0] == f.min() and got[2] == f.max() and got[3] == 2
    assert abs(got[1] - f.mean()) <= 1e-12 * np.abs(f).max()
    y = torch.tensor(state(o, 51), dtype=torch.float32, device="cuda").reshape(-1)
    pv = m._param_vector(y.device)
    for engine, want in (("stages", {0: 3 * 6, 2: 0}), ("cluster", {0: 0, 2: 1})):
        pl.set_engine(engine)
        pl.set_profiling(True)
        pl.step(y, pv, 5.0, 3, "tsit5", True)
        torch.cuda.synchronize()
        for k, launches in want.items():
            ms, cnt = pl.kernel_stats(_lib.K["QG_SWM_K_STAGE"] if k == 0 else _lib.K["QG_SWM_K_CLUSTER"])
            assert cnt == launches and (ms > 0) == (launches > 0), (engine, k, cnt, ms)
        pl.set_profiling(False)
    assert pl.status() == 0


def test_plan_argument_checks():
    """The plan's calls take the parameters as any 3-value sequence (moved to the plan's device as
    float32) and refuse, before any launch, a state on the host, of the wrong size or on another
    device, and a parameter vector of the wrong length."""
    m, o = pair((16, 16), (500.0, 500.0), (9.81, 0.02), "wall")
    y = torch.tensor(state(o, 3), dtype=torch.float32, device="cuda").reshape(-1)
    plan = m.plan(y.device)
    pv = m._param_vector(y.device)
    ref = plan.rhs(y, pv, True)
    torch.testing.assert_close(plan.rhs(y, [float(v) for v in pv.cpu()], True), ref, rtol=0, atol=0)
    torch.testing.assert_close(plan.rhs(y, pv.double().cpu(), True), ref, rtol=0, atol=0)
    with pytest.raises(ValueError):
        plan.rhs(y, pv[:2], True)
    with pytest.raises(ValueError):
        plan.step(y.clone(), torch.zeros(4, device="cuda"), 10.0, 1, "heun", True)
    with pytest.raises(TypeError):
        plan.rhs(y.cpu(), pv, True)
    with pytest.raises(ValueError):
        plan.rhs(y[:-1], pv, True)
    with pytest.raises(ValueError):
        plan.rhs(y, pv, True, out=torch.empty(y.numel() - 1, device="cuda"))
    with pytest.raises(TypeError):
        plan.field_stats(y.cpu())
