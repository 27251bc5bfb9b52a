"""The persistent step kernel's bounded grid barrier, made to run out on purpose.

The runner of the reference stops on a diverged state (``somax/_src/cli/_run.py:671-686``); the
device-side counterpart here is the status word that ``qg_status`` reads.  With a wait limit of
a few dozen clock cycles, the CTAs of a persistent launch give up at the first grid barrier
that does not fill at once: every CTA drains its copies in flight, frees its tensor memory and
returns, and ``qg_status`` reports QG_ERR_TIMEOUT.  Nothing faults and nothing hangs, so the
context stays usable: the next call, with the default limit restored, must again match the
float64 oracle (1e-5 relative L2 after 10 SSP-RK3 steps) and the multi-launch path (1e-6), which
also checks that the arrivals the aborted launch left at the barrier are cleared.
"""

import numpy as np
import pytest
import torch

import somax_gb300 as sg
from oracle import qg as O
from somax_gb300 import _lib
from somax_gb300 import testcases as tc

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = a.detach().cpu().double().numpy()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_grid_barrier_timeout_is_reported_and_recovered():
    cfg = tc.C2
    kw = cfg.model_kwargs()
    m = sg.BaroclinicQG.create(**kw, precision="bf16x3", persistent=True, cluster=False)
    plan = m.plan()
    q0 = tc.initial_pv(cfg, seed=3)
    qd = torch.tensor(q0, dtype=torch.float32, device="cuda")
    assert plan.launches_per_call(2, "ssprk3") == 3  # pack, the persistent kernel, unpack

    plan.set_wait_limit(32)
    m.step(sg.BaroclinicQGState(q=qd.clone()), cfg.dt, 2, cfg.scheme)
    torch.cuda.synchronize()
    assert plan.status() == _lib.K["QG_ERR_TIMEOUT"]
    assert plan.status() == 0  # qg_status cleared the flag

    plan.set_wait_limit(0)
    q10 = m.step(sg.BaroclinicQGState(q=qd.clone()), cfg.dt, 10, cfg.scheme).q
    assert plan.status() == 0
    o = O.baroclinic_model(nx=cfg.n, ny=cfg.n, Lx=cfg.L, Ly=cfg.L, f0=kw["f0"], beta=kw["beta"], H=cfg.H,
                           g_prime=cfg.g_prime, bottom_drag=cfg.bottom_drag, wind_amplitude=kw["wind_amplitude"],
                           biharmonic_viscosity=cfg.biharmonic_viscosity)
    r10 = O.integrate(o, q0, cfg.dt, 10, cfg.scheme)
    assert rel(q10[:, 1:-1, 1:-1], r10[:, 1:-1, 1:-1]) < 1e-5

    g = sg.BaroclinicQG.create(**kw, precision="bf16x3", persistent=False, cluster=False)
    g10 = g.step(sg.BaroclinicQGState(q=qd.clone()), cfg.dt, 10, cfg.scheme).q
    assert rel(q10, g10.cpu().double().numpy()) < 1e-6


def test_wait_limit_rejects_negative():
    cfg = tc.C2
    m = sg.BaroclinicQG.create(**dict(cfg.model_kwargs(), nx=32, ny=32), precision="bf16x3", persistent=True)
    with pytest.raises(_lib.QGError):
        m.plan().set_wait_limit(-1)
