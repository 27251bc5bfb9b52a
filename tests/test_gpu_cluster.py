"""Cluster-resident stepping (qg_options.cluster): one thread-block cluster per member runs
every stage of every step of a ``step`` call in one launch, FP32 DST-I passes on the CUDA
cores with the state in shared memory.  Checked against the float64 oracle and against the
multi-launch FP32 path on the same inputs (Heun and SSP-RK3, baroclinic and barotropic,
square and rectangular grids, identical-member ensembles, the BC flag and chunked calls)."""

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


def pair(nx, ny, nl, seed, barotropic=False):
    kw = dict(lateral_viscosity=60.0, bottom_drag=1e-7, wind_amplitude=1e-10, biharmonic_viscosity=1e9)
    if barotropic:
        m = sg.BarotropicQG.create(nx=nx, ny=ny, Lx=1.2e6, Ly=1e6, **kw)
        o = O.barotropic_model(nx=nx, ny=ny, Lx=1.2e6, Ly=1e6, **kw)
        nl = 1
    else:
        H = (400.0, 1100.0, 2600.0, 900.0, 1500.0)[:nl] if nl > 1 else (4000.0,)
        g = (9.81, 0.025, 0.0125, 0.01, 0.008)[:nl] if nl > 1 else (0.0055,)
        m = sg.BaroclinicQG.create(nx=nx, ny=ny, Lx=1.2e6, Ly=1e6, n_layers=nl, H=H, g_prime=g, **kw)
        o = O.baroclinic_model(nx=nx, ny=ny, Lx=1.2e6, Ly=1e6, H=H, g_prime=g, **kw)
    rng = np.random.default_rng(seed)
    q = tc.kminus3_field(max(nx, ny), seed, nl)[:, : ny + 2, : nx + 2] * 1e-6
    q = q + 1e-7 * rng.standard_normal(q.shape)  # a non-zero ring too
    if barotropic:
        q = q[0]
    return m, o, q


SHAPES = [(17, 13, 3, False), (30, 30, 1, False), (64, 40, 5, False), (28, 28, 1, True), (128, 128, 3, False),
          (100, 70, 2, False)]


@pytest.mark.parametrize("nx,ny,nl,bt", SHAPES)
def test_cluster_steps_against_oracle(nx, ny, nl, bt):
    m, o, q = pair(nx, ny, nl, 70 + nl, bt)
    plan = sg.Plan([m.spec], "fp32", cluster=True)
    assert plan.engine()["cluster_ctas"] >= 2
    ref_plan = sg.Plan([m.spec], "fp32", cluster=False)
    assert ref_plan.engine()["cluster_ctas"] == 0
    pv = m._param_vector(torch.device("cuda"))
    qd = torch.tensor(q, dtype=torch.float32, device="cuda")
    for scheme in ("heun", "ssprk3"):
        got = plan.step(qd.clone(), pv, 1200.0, 3, scheme)
        assert plan.status() == 0
        assert rel(got, O.integrate(o, q, 1200.0, 3, scheme)) < RTOL_STEP
        assert rel(got, ref_plan.step(qd.clone(), pv, 1200.0, 3, scheme)) < 1e-6


@pytest.mark.parametrize("apply_bc", [True, False])
def test_cluster_bc_flag_and_chunks(apply_bc):
    """The ring of the state is zeroed only with the flag; every stage input reads a zero
    ring; two calls of n steps without the flag equal one call of 2n."""
    m, o, q = pair(40, 33, 3, 5)
    pv = m._param_vector(torch.device("cuda"))
    plan = sg.Plan([m.spec], "fp32", cluster=True)
    ref = sg.Plan([m.spec], "fp32", cluster=False)
    qd = torch.tensor(q, dtype=torch.float32, device="cuda")
    a = plan.step(qd.clone(), pv, 1200.0, 4, "ssprk3", apply_bc=apply_bc)
    b = ref.step(qd.clone(), pv, 1200.0, 4, "ssprk3", apply_bc=apply_bc)
    assert rel(a, b) < 1e-6
    c = plan.step(plan.step(qd.clone(), pv, 1200.0, 2, "ssprk3", apply_bc=apply_bc), pv, 1200.0, 2, "ssprk3",
                  apply_bc=False)
    assert rel(c, a) < 1e-6


def test_cluster_ensemble_of_identical_members():
    """One cluster per member: three 3-layer 48 x 36 members with their own states and winds."""
    models, qs, os = [], [], []
    H, g = (400.0, 1100.0, 2600.0), (9.81, 0.025, 0.0125)
    for i in range(3):
        _, _, q = pair(48, 36, 3, 90 + i)
        kw = dict(lateral_viscosity=60.0, bottom_drag=1e-7, wind_amplitude=1e-10 * (1 + i), biharmonic_viscosity=1e9)
        m = sg.BaroclinicQG.create(nx=48, ny=36, Lx=1.2e6, Ly=1e6, n_layers=3, H=H, g_prime=g, **kw)
        o = O.baroclinic_model(nx=48, ny=36, Lx=1.2e6, Ly=1e6, H=H, g_prime=g, **kw)
        models.append(m)
        qs.append(q)
        os.append(o)
    ens = sg.QGEnsemble(models, precision="fp32", cluster=True)
    assert ens.plan.engine()["cluster_ctas"] >= 2
    packed = ens.pack([torch.tensor(q, dtype=torch.float32, device="cuda") for q in qs])
    ens.step(packed, 1200.0, 3, "ssprk3")
    assert ens.plan.status() == 0
    for got, o, q in zip(ens.unpack(packed), os, qs):
        assert rel(got, O.integrate(o, q, 1200.0, 3, "ssprk3")) < RTOL_STEP


def test_cluster_not_used_for_unlike_or_masked_members():
    m1, _, _ = pair(30, 30, 3, 1)
    m2, _, _ = pair(40, 30, 3, 2)
    assert sg.Plan([m1.spec, m2.spec], "fp32", cluster=True).engine()["cluster_ctas"] == 0
    mask = np.ones((32, 32), np.uint8)
    mask[10:14, 10:14] = 0
    mm = sg.BaroclinicQG.create(nx=30, ny=30, Lx=1.2e6, Ly=1e6, mask=mask)
    assert sg.Plan([mm.spec], "fp32", cluster=True).engine()["cluster_ctas"] == 0
