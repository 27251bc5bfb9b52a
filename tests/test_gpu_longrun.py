"""Long runs judged by energy and enstrophy statistics.

The flow of a wind-driven double gyre becomes chaotic, so after many steps two correct
integrations (float32 on the GPU, float64 on the host) need not agree point by point; what
must agree are the statistics of its kinetic energy and enstrophy (``BaroclinicQG.diagnose``,
``baroclinic.py:197-228``, on the GPU ``qg_diagnose``; on the host ``oracle.qg.diagnose``).

* Configuration 1, the barotropic 64^2 double gyre (Rd = 50 km, Heun, dt = 4000 s), for one
  model year (7884 steps), sampled every 219 steps.
* Configuration 2, the 3-layer 128^2 double gyre (SSP-RK3, dt = 1200 s) on the split-BF16x3
  tensor-core path, for 30 model days (2160 steps), sampled every 72 steps (one model day).

Bounds: the time means of total KE and of total enstrophy within 1 % of the float64 run's,
and every sample's KE within 5 %.  The measured differences are printed with the ``LONGRUN:``
prefix.
"""

import numpy as np
import pytest
import torch

import somax_gb300 as sg
from oracle import qg as O
from somax_gb300 import testcases as tc

pytestmark = pytest.mark.gpu


def oracle_model(cfg):
    kw = cfg.model_kwargs()
    return O.baroclinic_model(nx=cfg.n, ny=cfg.n, Lx=cfg.L, Ly=cfg.L, f0=kw["f0"], beta=kw["beta"], H=cfg.H,
                              g_prime=cfg.g_prime, lateral_viscosity=cfg.lateral_viscosity,
                              bottom_drag=cfg.bottom_drag, wind_amplitude=kw["wind_amplitude"],
                              biharmonic_viscosity=cfg.biharmonic_viscosity)


def series(cfg, precision, n_samples, every):
    m = sg.BaroclinicQG.create(**cfg.model_kwargs(), precision=precision)
    o = oracle_model(cfg)
    q0 = tc.initial_pv(cfg, seed=0).astype(np.float32).astype(np.float64)
    q = torch.tensor(q0, dtype=torch.float32, device="cuda")
    gke, gen = [], []
    for k in range(n_samples):
        q = m.step(sg.BaroclinicQGState(q=q), cfg.dt, every, cfg.scheme, apply_bc=(k == 0)).q
        d = m.diagnose(sg.BaroclinicQGState(q=q))
        gke.append(float(d.total_kinetic_energy))
        gen.append(float(d.total_enstrophy))
    assert m.plan().status() == 0
    O.set_workers(16)
    r = O.apply_boundary_conditions(o, q0)
    oke, oen = [], []

    def f(y):
        return O.vector_field(o, O.apply_boundary_conditions(o, y))

    for k in range(n_samples):
        for _ in range(every):
            r = O.rk_step(f, r, cfg.dt, cfg.scheme)
        d = O.diagnose(o, r)
        oke.append(float(d["total_kinetic_energy"]))
        oen.append(float(d["total_enstrophy"]))
    O.set_workers(1)
    return np.array(gke), np.array(gen), np.array(oke), np.array(oen), q.cpu().double().numpy(), r


@pytest.mark.parametrize("case", ["c1_one_year", "c2_30_days_bf16x3"])
def test_long_run_statistics(case):
    if case == "c1_one_year":
        cfg, precision, n_samples, every = tc.C1, "fp32", 36, 219
    else:
        cfg, precision, n_samples, every = tc.C2, "bf16x3", 30, 72
    gke, gen, oke, oen, qg, qo = series(cfg, precision, n_samples, every)
    d_ke = abs(gke.mean() - oke.mean()) / oke.mean()
    d_en = abs(gen.mean() - oen.mean()) / oen.mean()
    d_sample = float(np.max(np.abs(gke - oke) / oke))
    s = (Ellipsis, slice(1, -1), slice(1, -1))
    e_end = float(np.linalg.norm(qg[s] - qo[s]) / np.linalg.norm(qo[s]))
    print(f"LONGRUN: {case}: time-mean KE rel diff {d_ke:.2e}, time-mean enstrophy rel diff {d_en:.2e}, "
          f"max per-sample KE rel diff {d_sample:.2e}, final-state interior rel L2 {e_end:.2e}, "
          f"KE {oke[0]:.3e} -> {oke[-1]:.3e}")
    assert np.all(np.isfinite(gke)) and np.all(np.isfinite(gen))
    assert d_ke < 1e-2 and d_en < 1e-2
    assert d_sample < 5e-2
