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


def _dense_jacobian(f, x, h=1e-7):
    """Columns (f(x + h e_j) - f(x - h e_j)) / 2h: exact up to rounding for the masked RHS
    (quadratic in q) and the masked inversion (linear)."""
    x = np.asarray(x, np.float64)
    cols = []
    for j in range(x.size):
        e = np.zeros(x.size)
        e[j] = h
        cols.append(((f((x.ravel() + e).reshape(x.shape)) - f((x.ravel() - e).reshape(x.shape))) / (2 * h)).ravel())
    return np.stack(cols, axis=1)


@pytest.mark.parametrize("barotropic,apply_bc", [(False, True), (False, False), (True, True)])
@pytest.mark.parametrize("precision", ["fp32", "bf16x3"])
def test_masked_rhs_vjp_dense(barotropic, apply_bc, precision):
    """qg_rhs_vjp of a masked member against the transposed dense Jacobian of the float64 masked
    RHS (land rules: q read as 0, psi = 0, dq = 0 and lap q = 0 on land; the capacitance
    correction around the DST solve), and the parameter cotangents against the float64
    parameter derivatives.  RTOL_MASK (the masked inversion's FP32 floor)."""
    nx, ny, nl = 20, 16, 1 if barotropic else 2
    mask = tc.land_mask(ny, nx, frac=0.15, seed=4)
    m, o = pair(nx, ny, nl, mask, precision, barotropic=barotropic)
    shape = m.shape
    q = field((nl, ny + 2, nx + 2), 8).reshape(shape)
    g = np.random.default_rng(9).standard_normal(shape)
    q32 = q.astype(np.float32).astype(np.float64)

    def F(x):
        xx = O.apply_boundary_conditions(o, x) if apply_bc else x
        return OM.vector_field(o, xx, mask)

    Jt_g = _dense_jacobian(F, q32, h=float(np.abs(q32).max())).T @ g.ravel()
    pv = m._param_vector(torch.device("cuda"))
    qb, pb = m.plan().rhs_vjp(cuda(q32).reshape(-1), pv, cuda(g).reshape(-1), apply_bc=apply_bc)
    assert m.plan().status() == 0
    assert rel(qb, Jt_g) < RTOL_MASK
    # parameters: the RHS is affine in each of them
    names = ("lateral_viscosity", "bottom_drag", "wind_amplitude", "biharmonic_viscosity")
    base = F(q32)
    xx = O.apply_boundary_conditions(o, q32) if apply_bc else q32
    for k, name in enumerate(names):
        val = float(getattr(o, name))
        # affine in each parameter: any step is exact; size it so the change is 1e3 |rhs|
        g1 = OM.vector_field(o, xx, mask, params={name: val + 1.0}) - base
        h = 1e3 * float(np.linalg.norm(base)) / max(float(np.linalg.norm(g1)), 1e-300)
        d = (OM.vector_field(o, xx, mask, params={name: val + h}) - base) / h
        ref = float(np.sum(d * g))
        if abs(ref) > 0:
            assert abs(float(pb[k]) - ref) <= 1e-3 * abs(ref), (name, float(pb[k]), ref)


@pytest.mark.parametrize("precision,refine", [("fp32", 0), ("bf16x3", 1)])
def test_masked_invert_vjp_dense(precision, refine):
    """qg_invert_vjp of a masked member is the transposed dense matrix of the masked inversion
    (the map is symmetric: the adjoint runs the same capacitance-corrected solve)."""
    nx, ny, nl = 18, 15, 2
    mask = tc.land_mask(ny, nx, frac=0.15, seed=11)
    m, o = pair(nx, ny, nl, mask, precision, refine=refine)
    shape = m.shape
    g = np.random.default_rng(12).standard_normal(shape)
    At_g = _dense_jacobian(lambda x: OM.invert_pv(o, x, mask), np.zeros(shape), h=1.0).T @ g.ravel()
    qb = m.plan().invert_vjp(cuda(g).reshape(-1))
    assert m.plan().status() == 0
    assert rel(qb, At_g) < RTOL_MASK


def test_masked_integrate_gradient_vs_float64_differences():
    """Gradient through 5 SSP-RK3 steps of a masked 3-layer basin (checkpoints every 2) along a
    random direction of q0 and in tau0, against float64 central differences of the masked
    oracle (1e-3)."""
    nx, ny, nl = 24, 20, 3
    mask = tc.land_mask(ny, nx, frac=0.15, seed=13)
    m, o = pair(nx, ny, nl, mask, "bf16x3")
    q0 = np.where(OM.land(mask), 0.0, field((nl, ny + 2, nx + 2), 14)).astype(np.float32).astype(np.float64)
    w = np.random.default_rng(15).standard_normal(q0.shape)
    d = np.where(OM.land(mask), 0.0, np.random.default_rng(16).standard_normal(q0.shape)) * 1e-6
    dt, n = 1200.0, 5
    tau = float(o.wind_amplitude)

    qt = cuda(q0).requires_grad_(True)
    m.params = sg.QGParams(torch.tensor(60.0), torch.tensor(1e-7), torch.tensor(tau, requires_grad=True),
                           torch.tensor(1e9))
    sol = m.integrate(sg.BaroclinicQGState(q=qt), 0.0, n * dt, dt, solver="ssprk3", checkpoint_every=2)
    loss = (sol.ys.q[-1].double() * torch.tensor(w, device="cuda")).sum()
    loss.backward()
    gd = float((qt.grad.double().cpu().numpy() * d).sum())
    gtau = float(m.params.wind_amplitude.grad)

    def L(q, t):
        import dataclasses
        oo = dataclasses.replace(o, wind_amplitude=t)
        return float(np.sum(OM.integrate(oo, q, mask, dt, n, "ssprk3") * w))

    eps = 1e-3
    fd = (L(q0 + eps * d, tau) - L(q0 - eps * d, tau)) / (2 * eps)
    fdt = (L(q0, tau * (1 + eps)) - L(q0, tau * (1 - eps))) / (2 * eps * tau)
    assert abs(gd - fd) <= 1e-3 * abs(fd), (gd, fd)
    assert abs(gtau - fdt) <= 1e-3 * abs(fdt), (gtau, fdt)
