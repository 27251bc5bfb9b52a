"""The persistent step kernel and multi-member plans (ensembles) against the per-member
multi-launch path and the float64 oracle."""

import numpy as np
import pytest
import torch

import somax_gb300 as sg
from oracle import qg as O
from somax_gb300 import testcases as tc

pytestmark = pytest.mark.gpu

RTOL_STEP = 1e-5


def rel(a, b):
    a = a.detach().cpu().double().numpy() if isinstance(a, torch.Tensor) else a
    b = b.detach().cpu().double().numpy() if isinstance(b, torch.Tensor) else b
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def member(n, nl, seed, precision="bf16x3", persistent=True, nu4=1e9, tau=1e-10):
    H = (400.0, 1100.0, 2600.0, 900.0, 1500.0)[:nl] if nl > 1 else (4000.0,)
    g = (9.81, 0.025, 0.0125, 0.01, 0.008)[:nl] if nl > 1 else (0.0055,)
    m = sg.BaroclinicQG.create(nx=n[0], ny=n[1], Lx=2e6, Ly=1.8e6, n_layers=nl, H=H, g_prime=g,
                               lateral_viscosity=50.0, bottom_drag=1e-7, wind_amplitude=tau,
                               biharmonic_viscosity=nu4, precision=precision, persistent=persistent,
                               cluster=False)
    o = O.baroclinic_model(nx=n[0], ny=n[1], Lx=2e6, Ly=1.8e6, H=H, g_prime=g, lateral_viscosity=50.0,
                           bottom_drag=1e-7, wind_amplitude=tau, biharmonic_viscosity=nu4)
    k = tc.kminus3_field(max(n), seed, nl)[:, : n[1] + 2, : n[0] + 2] * 1e-6
    return m, o, k


@pytest.mark.parametrize("precision", ["bf16x3", "tf32"])
@pytest.mark.parametrize("scheme", ["heun", "ssprk3"])
def test_persistent_equals_multi_launch(precision, scheme):
    mp, _, q = member((40, 33), 3, 1, precision, persistent=True)
    mg, _, _ = member((40, 33), 3, 1, precision, persistent=False)
    qd = torch.tensor(q, dtype=torch.float32, device="cuda")
    a = mp.step(sg.BaroclinicQGState(q=qd), 1200.0, 5, scheme).q
    b = mg.step(sg.BaroclinicQGState(q=qd), 1200.0, 5, scheme).q
    assert mp.plan().status() == 0
    assert rel(a, b) < 1e-6


def test_persistent_config2_10_steps_vs_oracle():
    cfg = tc.C2
    kw = cfg.model_kwargs()
    m = sg.BaroclinicQG.create(**kw, precision="bf16x3", persistent=True)
    o = O.baroclinic_model(nx=cfg.n, ny=cfg.n, Lx=cfg.L, Ly=cfg.L, f0=kw["f0"], beta=kw["beta"], H=cfg.H,
                           g_prime=cfg.g_prime, bottom_drag=cfg.bottom_drag, wind_amplitude=kw["wind_amplitude"],
                           biharmonic_viscosity=cfg.biharmonic_viscosity)
    q0 = tc.initial_pv(cfg, seed=0)
    q10 = m.step(sg.BaroclinicQGState(q=torch.tensor(q0, dtype=torch.float32, device="cuda")), cfg.dt, 10,
                 cfg.scheme).q
    assert m.plan().status() == 0
    r10 = O.integrate(o, q0, cfg.dt, 10, cfg.scheme)
    assert rel(q10[:, 1:-1, 1:-1], r10[:, 1:-1, 1:-1]) < RTOL_STEP


SPECS = [((30, 30), 1, 3), ((40, 33), 3, 4), ((24, 24), 5, 5), ((130, 66), 2, 6), ((17, 13), 3, 7)]


@pytest.mark.parametrize("precision,persistent", [("bf16x3", True), ("bf16x3", False), ("fp32", False)])
def test_ensemble_matches_members(precision, persistent):
    ms, qs = [], []
    for n, nl, seed in SPECS:
        m, _, q = member(n, nl, seed, precision, persistent)
        ms.append(m)
        qs.append(torch.tensor(q, dtype=torch.float32, device="cuda"))
    ens = sg.QGEnsemble(ms, precision=precision, persistent=persistent)
    packed = ens.pack(qs)
    # rhs and inversion member by member
    dq = ens.unpack(ens.rhs(packed))
    psi = ens.unpack(ens.invert(packed))
    for m, q, d, p in zip(ms, qs, dq, psi):
        assert rel(d, m.vector_field(0.0, sg.BaroclinicQGState(q=q)).q) < 1e-6
        assert rel(p, m._invert_pv(q)) < 1e-6
    # stepping all members at once equals stepping each alone
    ens.step(packed, 1200.0, 4, "ssprk3")
    assert ens.plan.status() == 0
    for m, q, got in zip(ms, qs, ens.unpack(packed)):
        ref = m.step(sg.BaroclinicQGState(q=q), 1200.0, 4, "ssprk3").q
        assert rel(got, ref) < 1e-6


def test_ensemble_against_oracle():
    ms, qs, os = [], [], []
    for n, nl, seed in SPECS[:3]:
        m, o, q = member(n, nl, seed)
        ms.append(m)
        os.append(o)
        qs.append(q)
    ens = sg.QGEnsemble(ms, precision="bf16x3")
    packed = ens.pack([torch.tensor(q, dtype=torch.float32, device="cuda") for q in qs])
    ens.step(packed, 1200.0, 3, "ssprk3")
    for o, q, got in zip(os, qs, ens.unpack(packed)):
        ref = O.integrate(o, q, 1200.0, 3, "ssprk3")
        assert rel(got, ref) < RTOL_STEP


def test_ensemble_parameters_per_member():
    # members differ only in wind amplitude: each gets its own parameter vector
    m1, _, q = member((20, 20), 2, 9, tau=1e-10)
    m2, _, _ = member((20, 20), 2, 9, tau=3e-10)
    ens = sg.QGEnsemble([m1, m2], precision="bf16x3")
    qd = torch.tensor(q, dtype=torch.float32, device="cuda")
    d1, d2 = ens.unpack(ens.rhs(ens.pack([qd, qd])))
    assert rel(d1, m1.vector_field(0.0, sg.BaroclinicQGState(q=qd)).q) < 1e-6
    assert rel(d2, m2.vector_field(0.0, sg.BaroclinicQGState(q=qd)).q) < 1e-6
    assert rel(d1, d2) > 1e-3


def test_parallel_sweep_branches_bitwise_equal_serial():
    """The layer-per-warp sweep's (layer count, strip class) launches forked as parallel graph
    branches give the same bits as the same launches one after another: twenty groups (1-5
    layers, interior strips and the three kinds of edge strip), so that nineteen side branches
    share the plan's four side streams,
    stepped 19 steps (two replays of the eight-step graph with programmatic dependent launch
    across the join, then three of the one-step graph)."""
    specs = [((130, 98), 1, 21), ((130, 98), 2, 22), ((190, 150), 3, 23), ((130, 130), 4, 24), ((200, 140), 5, 25)]
    ms, qs = [], []
    for n, nl, seed in specs:
        m, _, q = member(n, nl, seed, "bf16x3", persistent=False)
        ms.append(m)
        qs.append(torch.tensor(q, dtype=torch.float32, device="cuda"))
    ens = sg.QGEnsemble(ms, precision="bf16x3", persistent=False, stencil="lsweep32", cluster=False)
    groups = {(m.spec.n_layers, c) for m in ms for c in sg.qg.lsweep_classes(m.spec, 32)}
    assert len(groups) == 20
    q0 = ens.pack(qs)
    a = q0.clone()
    ens.step(a, 1200.0, 19, "ssprk3")
    ens.plan.set_parallel_sweep(False)
    b = q0.clone()
    ens.step(b, 1200.0, 19, "ssprk3")
    ens.plan.set_parallel_sweep(True)
    c = q0.clone()
    ens.step(c, 1200.0, 19, "ssprk3")
    assert ens.plan.status() == 0
    assert torch.isfinite(a).all()
    assert torch.equal(a, b)
    assert torch.equal(a, c)


def test_member_groups_bitwise_equal_one_plan():
    """An ensemble split into three plans stepped concurrently on their own streams (groups=3)
    gives the bits of the one-plan ensemble when the stencil variant and tile width are forced:
    every member's arithmetic is its own, whatever plan it sits in."""
    specs = [((64, 64), 1, 31), ((64, 64), 1, 32), ((128, 96), 3, 33), ((96, 80), 3, 34), ((60, 50), 5, 35),
             ((40, 33), 2, 36)]
    ms, qs = [], []
    for n, nl, seed in specs:
        m, _, q = member(n, nl, seed, "bf16x3", persistent=False)
        ms.append(m)
        qs.append(torch.tensor(q, dtype=torch.float32, device="cuda"))
    kw = dict(precision="bf16x3", persistent=False, stencil="lsweep32", gemm_tile=144, cluster=False)
    one = sg.QGEnsemble(ms, **kw)
    three = sg.QGEnsemble(ms, groups=3, **kw)
    assert len(three.plan.plans) == 3 and three.offsets == one.offsets
    a = one.pack(qs)
    b = a.clone()
    one.step(a, 1200.0, 11, "ssprk3")
    three.step(b, 1200.0, 11, "ssprk3")
    assert one.plan.status() == 0 and three.plan.status() == 0
    assert torch.equal(a, b)
    assert torch.equal(one.rhs(one.pack(qs)), three.rhs(three.pack(qs)))
