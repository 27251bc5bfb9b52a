"""Masked basins (land mask + FP64 capacitance correction) against the oracle's direct sparse
solve of the same discrete problem (``oracle/masked.py``), through the model API and the C ABI.

Tolerances (relative L2 against float64): inversion and RHS RTOL_MASK = 1e-4 (the FP32 DST
solve's error passes through the capacitance correction), three steps RTOL_STEP = 1e-5.
"""

import numpy as np
import pytest
import torch

import somax_gb300 as sg
from oracle import masked as OM
from oracle import qg as O
from somax_gb300 import testcases as tc

pytestmark = pytest.mark.gpu

RTOL_MASK = 1e-4
RTOL_STEP = 1e-5


def rel(a, b):
    a = a.detach().cpu().double().numpy() if isinstance(a, torch.Tensor) else a
    b = b.detach().cpu().double().numpy() if isinstance(b, torch.Tensor) else b
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def cuda(x):
    return torch.tensor(np.asarray(x), dtype=torch.float32, device="cuda")


def pair(nx, ny, nl, mask, precision="fp32", barotropic=False, refine=0, stencil=None, **kw):
    p = dict(lateral_viscosity=60.0, bottom_drag=1e-7, wind_amplitude=1e-10, biharmonic_viscosity=1e9)
    p.update(kw)
    if barotropic:
        m = sg.BarotropicQG.create(nx=nx, ny=ny, Lx=1.2e6, Ly=1e6, precision=precision, refine=refine,
                                   stencil=stencil, mask=mask, **p)
        o = O.barotropic_model(nx=nx, ny=ny, Lx=1.2e6, Ly=1e6, **p)
    else:
        H = (400.0, 1100.0, 2600.0, 900.0)[:nl]
        g = (9.81, 0.025, 0.0125, 0.01)[:nl]
        m = sg.BaroclinicQG.create(nx=nx, ny=ny, Lx=1.2e6, Ly=1e6, n_layers=nl, H=H, g_prime=g, precision=precision,
                                   refine=refine, stencil=stencil, mask=mask, **p)
        o = O.baroclinic_model(nx=nx, ny=ny, Lx=1.2e6, Ly=1e6, H=H, g_prime=g, **p)
    return m, o


def field(shape, seed):
    nl = int(np.prod(shape[:-2])) if len(shape) > 2 else 1
    q = tc.kminus3_field(max(shape[-2], shape[-1]) - 2, seed, nl)[:, : shape[-2], : shape[-1]] * 1e-6
    return q.reshape(shape)


@pytest.mark.parametrize("precision,refine", [("fp32", 0), ("bf16x3", 0), ("bf16x3", 1)])
@pytest.mark.parametrize("nx,ny,nl", [(62, 50, 3), (40, 40, 1), (96, 70, 2)])
def test_masked_inversion(precision, refine, nx, ny, nl):
    mask = tc.land_mask(ny, nx, frac=0.15, seed=nx + nl)
    m, o = pair(nx, ny, nl, mask, precision, refine=refine)
    q = field((nl, ny + 2, nx + 2), 1)
    psi = m._invert_pv(cuda(q))
    ref = OM.invert_pv(o, q, mask)
    assert rel(psi, ref) < RTOL_MASK
    assert torch.all(psi[:, torch.as_tensor(OM.land(mask))] == 0)


def test_masked_barotropic_inversion_and_rhs():
    mask = tc.land_mask(50, 60, frac=0.15, seed=7)
    m, o = pair(60, 50, 1, mask, barotropic=True)
    q = field((52, 62), 2)
    assert rel(m._invert_pv(cuda(q)), OM.invert_pv(o, q, mask)) < RTOL_MASK
    dq = m.vector_field(0.0, sg.BarotropicQGState(q=cuda(q))).q
    assert rel(dq, OM.vector_field(o, q, mask)) < RTOL_MASK


@pytest.mark.parametrize("stencil", ["tile32x8", "tile64x16", "sweep16", "lsweep16"])
def test_masked_rhs_and_steps(stencil):
    nx, ny, nl = 70, 54, 3
    mask = tc.land_mask(ny, nx, frac=0.15, seed=3)
    m, o = pair(nx, ny, nl, mask, stencil=stencil)
    q = field((nl, ny + 2, nx + 2), 4)
    dq = m.vector_field(0.0, sg.BaroclinicQGState(q=cuda(q))).q
    assert rel(dq, OM.vector_field(o, q, mask)) < RTOL_MASK
    assert torch.all(dq[:, torch.as_tensor(OM.land(mask))] == 0)
    got = m.step(sg.BaroclinicQGState(q=cuda(q)), 1200.0, 3, "ssprk3").q
    assert m.plan().status() == 0
    assert rel(got, OM.integrate(o, q, mask, 1200.0, 3, "ssprk3")) < RTOL_STEP


def test_all_ocean_mask_is_the_unmasked_model():
    nx, ny = 40, 30
    mask = np.ones((ny + 2, nx + 2), np.uint8)
    mask[0] = mask[-1] = 0
    mask[:, 0] = mask[:, -1] = 0
    mm, _ = pair(nx, ny, 3, mask)
    mu, _ = pair(nx, ny, 3, None)
    q = cuda(field((3, ny + 2, nx + 2), 5))
    assert torch.equal(mm.vector_field(0.0, sg.BaroclinicQGState(q=q)).q,
                       mu.vector_field(0.0, sg.BaroclinicQGState(q=q)).q)


def test_ensemble_mixes_masked_and_open_members():
    specs = [((50, 40), 3, 0.15), ((30, 30), 1, 0.0), ((64, 48), 2, 0.2)]
    ms, os, qs, masks = [], [], [], []
    for k, ((nx, ny), nl, frac) in enumerate(specs):
        mask = tc.land_mask(ny, nx, frac=frac, seed=10 + k) if frac else None
        m, o = pair(nx, ny, nl, mask, "bf16x3")
        ms.append(m)
        os.append(o)
        masks.append(mask)
        qs.append(field((nl, ny + 2, nx + 2), 20 + k))
    ens = sg.QGEnsemble(ms, precision="bf16x3", persistent=True)
    packed = ens.pack([cuda(q) for q in qs])
    ens.step(packed, 1200.0, 3, "ssprk3")
    assert ens.plan.status() == 0
    for got, o, q, mask in zip(ens.unpack(packed), os, qs, masks):
        ref = OM.integrate(o, q, mask, 1200.0, 3, "ssprk3") if mask is not None else O.integrate(o, q, 1200.0, 3,
                                                                                                  "ssprk3")
        assert rel(got, ref) < RTOL_STEP


def test_masked_adjoint_is_refused():
    mask = tc.land_mask(20, 20, frac=0.15, seed=1)
    m, _ = pair(20, 20, 2, mask)
    q = cuda(field((2, 22, 22), 6))
    with pytest.raises(RuntimeError):
        m.plan().rhs_vjp(q, m._param_vector(torch.device("cuda")), q, apply_bc=True)
