"""Configuration C4: the full 256-member ragged ensemble against the float64 oracle.

The mix of the ensemble benchmark (96 one-layer 64^2 basins with a 50 km deformation radius,
96 three-layer 128^2, 48 three-layer 256^2 and 16 five-layer 256^2 double gyres, H of the
five-layer members geometric from 200 m to 2000 m, every member with its own seeded PV and a
wind amplitude drawn from 0.05-0.12 N/m^2; ``gfd_testcases.py:231-287`` is the factory of the
reference's double gyres) is built exactly as ``bench.py --config ensemble256`` builds it:
one plan, split-BF16x3 tensor-core DST passes, the autotuner left on so that it picks the
stencil, tile width and schedule the benchmark runs with.  After 10 SSP-RK3 steps at
dt = 1200 s every member's interior must be within 1e-5 relative L2 of its own float64
integration (``SomaxModel.integrate``, ``core/model.py:53-88``, restated in ``oracle.qg``).
Checking every member against the oracle also covers the per-member check: a member whose
result depended on its neighbours in the packed state would miss its own float64 run.

The 256 float64 integrations run in a pool of spawned processes (about a minute of CPU).
"""

import concurrent.futures as cf
import multiprocessing as mp
import os

import numpy as np
import pytest
import torch

import somax_gb300 as sg
from oracle import qg as O
from somax_gb300 import testcases as tc

pytestmark = pytest.mark.gpu

RTOL_10 = 1e-5
N_STEPS = 10


def oracle_kwargs(cfg, tau0):
    kw = tc.member_kwargs(cfg, tau0)
    return dict(nx=cfg.n, ny=cfg.n, Lx=cfg.L, Ly=cfg.L, f0=kw["f0"], beta=kw["beta"], H=tuple(cfg.H),
                g_prime=tuple(cfg.g_prime), lateral_viscosity=cfg.lateral_viscosity, bottom_drag=cfg.bottom_drag,
                wind_amplitude=kw["wind_amplitude"], biharmonic_viscosity=cfg.biharmonic_viscosity)


def test_c4_ensemble256_10_steps_every_member():
    members = tc.c4_members(seed=0)
    assert len(members) == 256
    models = [sg.BaroclinicQG.create(**tc.member_kwargs(cfg, tau0), precision="bf16x3", persistent=False)
              for cfg, tau0, _ in members]
    ens = sg.QGEnsemble(models, precision="bf16x3", persistent=False)
    q0s = [tc.initial_pv(cfg, seed=s).astype(np.float32) for cfg, _, s in members]
    packed = torch.tensor(np.concatenate([q.reshape(-1) for q in q0s]), device="cuda")
    dt, scheme = members[0][0].dt, members[0][0].scheme
    ens.step(packed, dt, N_STEPS, scheme)
    assert ens.plan.status() == 0
    tuning = ens.plan.tuning()
    print(f"C4: stencil {tuning['stencil']}, gemm tile {tuning['gemm_tile_n']}, engine {ens.plan.engine()}")
    got = [q.cpu().numpy() for q in ens.unpack(packed)]

    cases = [dict(model=oracle_kwargs(cfg, tau0), q0=q0, dt=dt, n_steps=N_STEPS, scheme=scheme, got=g)
             for (cfg, tau0, _), q0, g in zip(members, q0s, got)]
    workers = max(1, min(16, len(os.sched_getaffinity(0))))
    with cf.ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
        errs = list(ex.map(O.integrate_and_compare, cases, chunksize=4))

    worst = {}
    for (cfg, _, _), e in zip(members, errs):
        worst[cfg.name] = max(worst.get(cfg.name, 0.0), e)
    print("C4: worst 10-step interior rel L2 per class: " +
          ", ".join(f"{k} {v:.2e}" for k, v in worst.items()))
    assert set(worst) == {cfg.name for _, cfg in tc.C4_MIX}
    bad = [(i, e) for i, e in enumerate(errs) if not e < RTOL_10]
    assert not bad, bad[:8]
