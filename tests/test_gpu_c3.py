"""Configuration C3 without land: 3-layer 512^2 and 1024^2 double gyres, DST-I GEMMs in TF32
and in split-BF16x3 with FP32 accumulation, one FP32 residual-refinement sweep each.

Per precision mode and size, against the float64 oracle (``_invert_pv``,
``baroclinic.py:135-159``; ``SomaxModel.integrate``, ``core/model.py:53-88``):
* the inversion's relative L2 error per vertical mode, next to its FP32 floor: the same error
  of the float64 solution rounded to FP32 in layer space (the layer psi is stored in FP32, and
  its rounding, ~6e-8 of the barotropic mode's magnitude, projects onto the much smaller
  baroclinic modes as a relative error of 1e-6 to 2e-5);
* the Helmholtz relative residual ||q_m - (lap - lambda_m) psi_m|| / ||q_m|| per mode, next to
  its FP32 floor (the residual of the float64 solution rounded to FP32: rounding psi perturbs
  lap(psi) by ~1e-7 |psi| / dx^2, a large fraction of |q| for the barotropic mode at this size);
* the interior relative L2 of q after 10 SSP-RK3 steps at dt = 1200 s.

Measured on GB300 (modes 0, 1, 2):
* split-BF16x3 + refinement, 512^2: q after 10 steps 2.3e-7; psi 2.5e-7, 3.5e-6, 1.0e-5 against
  FP32 floors of 1.8e-8, 1.9e-6, 4.8e-6; residual 2.2x, 1.7x, 1.7x its floor.
* split-BF16x3 + refinement, 1024^2: q 3.1e-7; psi 1.4e-6, 8.2e-6, 2.1e-5 against FP32 floors of
  1.6e-8, 4.3e-6, 9.5e-6; residual 2.3x, 1.7x, 1.7x its floor.
* TF32 + refinement, 512^2: q 1.75e-5; psi 1.3e-3 (mode 0), 9.3e-6, 1.2e-5.
* TF32 + refinement, 1024^2: q 2.3e-4; psi 7.2e-3 (mode 0), 2.2e-5, 2.6e-5.

Bounds.  split-BF16x3 + refinement: psi per mode within 1e-5 or 3x its FP32 floor, residual 3x
its floor, q after 10 steps 1e-5 (the benchmark spec's bound).  TF32 + refinement does NOT meet the
spec 1e-5 at these sizes: the 10-bit mantissa leaves the barotropic mode's solve at
~1e-3 and one refinement sweep cannot remove it (its residual is computed in FP32, at the
floor above).  Its bounds are regression bounds a little above the measured values: psi mode 0
3e-3 / 1.5e-2 and q after 10 steps 5e-5 / 5e-4 at 512^2 / 1024^2.  Measured values are
printed with the ``C3:`` prefix.
"""

import numpy as np
import pytest
import torch

import somax_gb300 as sg
from oracle import qg as O
from somax_gb300 import testcases as tc

pytestmark = pytest.mark.gpu

BOUNDS = {  # (precision, n): (psi per mode, psi / its FP32 floor, residual / floor, q after 10 steps)
    ("bf16x3", 512): (1e-5, 3.0, 3.0, 1e-5),
    ("bf16x3", 1024): (1e-5, 3.0, 3.0, 1e-5),
    ("tf32", 512): (3e-3, None, None, 5e-5),
    ("tf32", 1024): (1.5e-2, None, None, 5e-4),
}
N_STEPS = 10
_CACHE = {}


def oracle_case(n):
    """float64 reference of one size: model, q0, psi(q0), q after 10 steps, floors."""
    if n in _CACHE:
        return _CACHE[n]
    cfg = tc.CONFIGS[f"baroclinic3_{n}"]
    kw = cfg.model_kwargs()
    o = O.baroclinic_model(nx=n, ny=n, Lx=cfg.L, Ly=cfg.L, f0=kw["f0"], beta=kw["beta"], H=cfg.H,
                           g_prime=cfg.g_prime, lateral_viscosity=cfg.lateral_viscosity,
                           bottom_drag=cfg.bottom_drag, wind_amplitude=kw["wind_amplitude"],
                           biharmonic_viscosity=cfg.biharmonic_viscosity)
    O.set_workers(16)
    q0 = tc.initial_pv(cfg, seed=0).astype(np.float32).astype(np.float64)
    psi = O.invert_pv(o, q0)
    q10 = O.integrate(o, q0, cfg.dt, N_STEPS, cfg.scheme)
    O.set_workers(1)
    _CACHE[n] = (cfg, o, q0, psi, q10)
    return _CACHE[n]


def modal_report(o, q, psi_got, psi_ref):
    g = o.grid
    lam = o.helmholtz_lambdas
    qm = o.modes.to_modal(q)
    pg, pr = o.modes.to_modal(psi_got), o.modes.to_modal(psi_ref)
    pf = o.modes.to_modal(psi_ref.astype(np.float32).astype(np.float64))
    s = (slice(2, -2), slice(2, -2))  # cells whose stencil stays off the ring

    def residual(x, k):
        r = qm[k] - O.helmholtz_apply_full(x, g.dx, g.dy, float(lam[k]))
        return float(np.linalg.norm(r[s]) / np.linalg.norm(qm[k][s]))

    def err(x, k):
        return float(np.linalg.norm(x[k] - pr[k]) / np.linalg.norm(pr[k]))

    return [(err(pg, k), err(pf, k), residual(pg[k], k), residual(pf[k], k)) for k in range(o.nl)]


@pytest.mark.parametrize("n", [512, 1024])
@pytest.mark.parametrize("precision", ["bf16x3", "tf32"])
def test_c3_unmasked(precision, n):
    cfg, o, q0, psi_ref, q10_ref = oracle_case(n)
    m = sg.BaroclinicQG.create(**cfg.model_kwargs(), precision=precision, refine=1)
    qd = torch.tensor(q0, dtype=torch.float32, device="cuda")
    psi = m._invert_pv(qd).cpu().double().numpy()
    rows = modal_report(o, q0, psi, psi_ref)
    q10 = m.step(sg.BaroclinicQGState(q=qd.clone()), cfg.dt, N_STEPS, cfg.scheme).q
    assert m.plan().status() == 0
    d = q10.cpu().double().numpy()[:, 1:-1, 1:-1] - q10_ref[:, 1:-1, 1:-1]
    e10 = float(np.linalg.norm(d) / np.linalg.norm(q10_ref[:, 1:-1, 1:-1]))
    print(f"C3: {precision} {n}^2 + 1 refinement: q 10-step rel L2 {e10:.2e}; per mode (psi rel L2, its FP32 "
          f"floor, residual, its FP32 floor): " +
          "; ".join(f"m{k} {e:.2e} {ef:.2e} {r:.2e} {f:.2e}" for k, (e, ef, r, f) in enumerate(rows)))
    emax, efac, rfac, qmax = BOUNDS[(precision, n)]
    for k, (err, err_floor, res, floor) in enumerate(rows):
        assert err < max(emax, (efac or 0.0) * err_floor), (k, err, err_floor)
        if rfac is not None:
            assert res < rfac * floor, (k, res, floor)
    assert e10 < qmax, e10
