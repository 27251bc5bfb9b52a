"""Parity of the hand-written adjoints (qg_rhs_vjp, qg_invert_vjp and the checkpointed RK
adjoint) with float64 derivatives of the oracle.

The reference takes these derivatives with JAX autodiff through ``integrate``
(``tests/models/test_qg_baroclinic.py:293-312``); the oracle gets them exactly from its
float64 forward (the RHS is quadratic in q and affine in the parameters, the inversion
linear) or, through many steps, by float64 central differences.

Tolerances (relative L2 against float64): the VJPs run in FP32 with the plan's DST
precision, so RTOL_VJP = 1e-4 (FP32 and split-BF16x3); gradients through 10-20 steps agree
with float64 central differences to RTOL_GRAD = 1e-3.  The C5 configuration (3-layer 256^2,
100 SSP-RK3 steps, checkpoints every 10) is checked against FP32 central differences on the
GPU with eps = 1e-3 relative along 20 random directions (RTOL_FD = 1e-2: the FP32 forward's
rounding, ~1e-6 of the loss, against a ~1e-3 change of the loss), and its tau0 gradient
against float64 central differences of the oracle (RTOL_GRAD).
"""

import numpy as np
import pytest
import torch

import somax_gb300 as sg
from oracle import adjoint as OA
from oracle import qg as O
from somax_gb300 import testcases as tc

pytestmark = pytest.mark.gpu

RTOL_VJP = 1e-4
RTOL_GRAD = 1e-3
RTOL_FD = 1e-2
PNAMES = OA.PARAM_NAMES


def rel(a, b):
    a = a.detach().cpu().double().numpy() if isinstance(a, torch.Tensor) else np.asarray(a, float)
    b = np.asarray(b, float)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def cuda(x):
    return torch.tensor(np.asarray(x), dtype=torch.float32, device="cuda")


def pair(nx, ny, nl, barotropic=False, precision="fp32", L=(1e6, 8e5), **p):
    kw = dict(lateral_viscosity=p.get("nu", 0.0), bottom_drag=p.get("kappa", 0.0),
              wind_amplitude=p.get("tau", 0.0), biharmonic_viscosity=p.get("nu4", 0.0))
    if barotropic:
        m = sg.BarotropicQG.create(nx=nx, ny=ny, Lx=L[0], Ly=L[1], precision=precision, **kw)
        o = O.barotropic_model(nx=nx, ny=ny, Lx=L[0], Ly=L[1], **kw)
    else:
        H = (400.0, 1100.0, 2600.0, 900.0, 1500.0)[:nl]
        g = (9.81, 0.025, 0.0125, 0.01, 0.008)[:nl]
        m = sg.BaroclinicQG.create(nx=nx, ny=ny, Lx=L[0], Ly=L[1], n_layers=nl, H=H, g_prime=g,
                                   precision=precision, **kw)
        o = O.baroclinic_model(nx=nx, ny=ny, Lx=L[0], Ly=L[1], H=H, g_prime=g, **kw)
    return m, o


def field(shape, seed, scale=1e-6):
    rng = np.random.default_rng(seed)
    nl = int(np.prod(shape[:-2])) if len(shape) > 2 else 1
    base = tc.kminus3_field(max(shape[-2], shape[-1]) - 2, seed, nl)[:, : shape[-2], : shape[-1]]
    return (base.reshape(shape) + 0.1 * rng.standard_normal(shape)) * scale


PHYS = dict(nu=80.0, kappa=1e-7, tau=1e-10, nu4=1e9)


@pytest.mark.parametrize("apply_bc", [False, True])
@pytest.mark.parametrize("nx,ny,nl,baro", [(10, 8, 3, False), (7, 9, 1, False), (9, 11, 1, True), (6, 6, 5, False)])
def test_rhs_vjp_dense(nx, ny, nl, baro, apply_bc):
    m, o = pair(nx, ny, nl, barotropic=baro, **PHYS)
    shape = (ny + 2, nx + 2) if baro else (nl, ny + 2, nx + 2)
    q = field(shape, 11)
    g = np.random.default_rng(12).standard_normal(shape)
    qb_ref, pb_ref = OA.rhs_vjp(o, q, g, apply_bc=apply_bc)
    plan = m.plan()
    qb, pb = plan.rhs_vjp(cuda(q), m._param_vector(torch.device("cuda")), cuda(g), apply_bc=apply_bc)
    assert rel(qb, qb_ref) < RTOL_VJP
    pb = pb.cpu().double().numpy()
    for k in range(4):
        assert abs(pb[k] - pb_ref[k]) <= RTOL_VJP * max(abs(pb_ref[k]), 1e-300), PNAMES[k]
    if apply_bc:
        qbn = qb.cpu().numpy().reshape(shape)
        assert np.all(qbn[..., 0, :] == 0) and np.all(qbn[..., :, -1] == 0)


@pytest.mark.parametrize("precision", ["fp32", "bf16x3"])
@pytest.mark.parametrize("nx,ny,nl", [(62, 62, 3), (40, 33, 5), (126, 126, 3)])
def test_rhs_vjp_dot_product(precision, nx, ny, nl):
    """<q_bar, d> = <g, J d> with J d exact from the oracle (any size)."""
    m, o = pair(nx, ny, nl, precision=precision, L=(2e6, 2e6), **PHYS)
    shape = (nl, ny + 2, nx + 2)
    q = field(shape, 13)
    rng = np.random.default_rng(14)
    g = rng.standard_normal(shape)
    plan = m.plan()
    qb, _ = plan.rhs_vjp(cuda(q), m._param_vector(torch.device("cuda")), cuda(g), apply_bc=True)
    qb = qb.cpu().double().numpy()
    for _ in range(3):
        d = field(shape, int(rng.integers(1 << 30)), scale=1.0)
        jd = OA.rhs_directional(o, q, d, apply_bc=True)
        lhs, ref = float(np.sum(qb * d)), float(np.sum(g * jd))
        # random d: the inner product averages the FP32 errors down, 10x RTOL_VJP is ample
        assert lhs == pytest.approx(ref, rel=10 * RTOL_VJP)


@pytest.mark.parametrize("precision", ["fp32", "bf16x3"])
def test_rhs_vjp_dense_tensor_core(precision):
    m, o = pair(14, 12, 3, precision=precision, **PHYS)
    q = field((3, 14, 16), 15)
    g = np.random.default_rng(16).standard_normal((3, 14, 16))
    qb_ref, pb_ref = OA.rhs_vjp(o, q, g, apply_bc=True)
    qb, pb = m.plan().rhs_vjp(cuda(q), m._param_vector(torch.device("cuda")), cuda(g), apply_bc=True)
    assert rel(qb, qb_ref) < RTOL_VJP
    assert rel(pb, pb_ref) < RTOL_VJP


@pytest.mark.parametrize("nx,ny,nl,baro", [(10, 8, 3, False), (9, 7, 1, True)])
def test_invert_vjp_dense(nx, ny, nl, baro):
    m, o = pair(nx, ny, nl, barotropic=baro)
    shape = (ny + 2, nx + 2) if baro else (nl, ny + 2, nx + 2)
    pb = np.random.default_rng(17).standard_normal(shape)
    ref = OA.invert_vjp(o, pb)
    got = m.plan().invert_vjp(cuda(pb))
    assert rel(got, ref) < RTOL_VJP


def test_autograd_through_the_model_api():
    """vector_field / _invert_pv as torch.autograd.Functions, gradients in q and params."""
    m, o = pair(12, 10, 3, **PHYS)
    q = field((3, 12, 14), 18)
    g = np.random.default_rng(19).standard_normal((3, 12, 14))
    m.params = sg.QGParams(*(torch.tensor(v, requires_grad=True) for v in (80.0, 1e-7, 1e-10, 1e9)))
    qt = cuda(q).requires_grad_(True)
    dq = m.vector_field(0.0, sg.BaroclinicQGState(q=qt)).q
    (dq * cuda(g)).sum().backward()
    qb_ref, pb_ref = OA.rhs_vjp(o, q, g)
    assert rel(qt.grad, qb_ref) < RTOL_VJP
    got = [float(t.grad) for t in (m.params.lateral_viscosity, m.params.bottom_drag, m.params.wind_amplitude,
                                   m.params.biharmonic_viscosity)]
    for k in range(4):
        assert abs(got[k] - pb_ref[k]) <= RTOL_VJP * abs(pb_ref[k]), PNAMES[k]
    qt2 = cuda(q).requires_grad_(True)
    psi = m._invert_pv(qt2)
    (psi * cuda(g)).sum().backward()
    assert rel(qt2.grad, OA.invert_vjp(o, g)) < RTOL_VJP


@pytest.mark.parametrize("scheme,n,every", [("ssprk3", 20, 5), ("heun", 12, 4), ("tsit5", 6, 4)])
def test_integrate_gradient_vs_float64_differences(scheme, n, every):
    """Loss 1/2 |psi_1(T) - target|^2 (the C5 loss) on a 3-layer 32^2 basin: gradient in q0
    and tau0 through model.integrate's checkpointed adjoint vs float64 central differences
    of the oracle."""
    tau = 1e-10
    m, o = pair(32, 32, 3, nu=100.0, kappa=1e-7, tau=tau, L=(1e6, 1e6))
    dt = 1200.0
    q0 = field((3, 34, 34), 21)
    target = 1.5 * O.invert_pv(o, field((3, 34, 34), 22))[0]
    m.params = sg.QGParams(*(torch.tensor(v, requires_grad=(i == 2)) for i, v in enumerate((100.0, 1e-7, tau, 0.0))))
    qt = cuda(q0).requires_grad_(True)
    sol = m.integrate(sg.BaroclinicQGState(q=qt), 0.0, n * dt, dt, solver=scheme, checkpoint_every=every)
    psi = m._invert_pv(sol.ys.q[-1])
    loss = 0.5 * ((psi[0].double() - torch.tensor(target, device="cuda")) ** 2).sum()
    loss.backward()
    gq = qt.grad.cpu().double().numpy()
    gtau = float(m.params.wind_amplitude.grad)

    def L_q(x):
        psi1 = O.invert_pv(o, OA.integrate(o, x, dt, n, scheme))[0]
        return 0.5 * float(np.sum((psi1 - target) ** 2))

    rng = np.random.default_rng(23)
    for _ in range(2):
        d = field((3, 34, 34), int(rng.integers(1 << 30)), scale=1.0)
        fd = OA.fd_directional(L_q, q0, d, rel=1e-4)
        assert float(np.sum(gq * d)) == pytest.approx(fd, rel=RTOL_GRAD)

    def L_tau(t):
        psi1 = O.invert_pv(o, OA.integrate(o, q0, dt, n, scheme, params={"wind_amplitude": float(t[0])}))[0]
        return 0.5 * float(np.sum((psi1 - target) ** 2))

    fd_tau = OA.fd_directional(L_tau, np.array([tau]), np.array([1.0]), rel=1e-3)
    assert gtau == pytest.approx(fd_tau, rel=RTOL_GRAD)


def test_c5_adjoint_vs_fp32_differences_20_directions():
    """C5: 3-layer 256^2, FP32, dt = 1200 s, 100 SSP-RK3 steps, checkpoints every 10, loss
    1/2 |psi_1(T) - target|^2 with a seeded target; gradients in q0 and tau0 against FP32
    central differences on the GPU (eps = 1e-3 relative, 20 seeded random directions drawn
    from the initial PV's k^-3 spectrum)."""
    cfg = tc.CONFIGS["baroclinic3_256"]
    kw = cfg.model_kwargs()
    m = sg.BaroclinicQG.create(**kw)
    tau = float(kw["wind_amplitude"])
    n, dt = 100, cfg.dt
    q0 = torch.tensor(tc.initial_pv(cfg, seed=0), dtype=torch.float32, device="cuda")
    rng = np.random.default_rng(31)
    target = m._invert_pv(torch.tensor(tc.initial_pv(cfg, seed=1), dtype=torch.float32, device="cuda"))[0].double()

    def loss_of(q, tau_v, grad=False):
        m.params = sg.QGParams(torch.tensor(kw["lateral_viscosity"]), torch.tensor(kw["bottom_drag"]),
                               torch.tensor(tau_v, requires_grad=grad), torch.tensor(kw["biharmonic_viscosity"]))
        sol = m.integrate(sg.BaroclinicQGState(q=q), 0.0, n * dt, dt, solver="ssprk3", checkpoint_every=10)
        psi = m._invert_pv(sol.ys.q[-1])
        return 0.5 * ((psi[0].double() - target) ** 2).sum()

    qt = q0.clone().requires_grad_(True)
    L = loss_of(qt, tau, grad=True)
    L.backward()
    gq = qt.grad.double()
    gtau = float(m.params.wind_amplitude.grad)
    errs = []
    with torch.no_grad():
        for k in range(20):
            # random directions with the spectrum of the initial PV (white noise lies where
            # the biharmonic damping and the inversion make the loss nearly flat)
            d = torch.tensor(tc.kminus3_field(cfg.n, int(rng.integers(1 << 30)), cfg.nl), dtype=torch.float32,
                             device="cuda")
            h = 1e-3 * float(q0.norm()) / float(d.norm())
            fd = (float(loss_of(q0 + h * d, tau)) - float(loss_of(q0 - h * d, tau))) / (2 * h)
            errs.append(abs(float((gq * d.double()).sum()) - fd) / max(abs(fd), 1e-300))
    assert max(errs) < RTOL_FD, errs
    # tau0 moves the loss by ~1e-4 of itself per 1e-3 step, under the FP32 forward's noise:
    # its central difference (eps = 1e-3 relative) runs on the float64 oracle instead
    o = O.baroclinic_model(nx=cfg.n, ny=cfg.n, Lx=cfg.L, Ly=cfg.L, f0=kw["f0"], beta=kw["beta"], H=cfg.H,
                           g_prime=cfg.g_prime, lateral_viscosity=kw["lateral_viscosity"],
                           bottom_drag=kw["bottom_drag"], wind_amplitude=tau,
                           biharmonic_viscosity=kw["biharmonic_viscosity"])
    q0n = q0.cpu().double().numpy()
    tgt = target.cpu().numpy()

    def L_tau(t):
        psi1 = O.invert_pv(o, OA.integrate(o, q0n, dt, n, "ssprk3", params={"wind_amplitude": float(t[0])}))[0]
        return 0.5 * float(np.sum((psi1 - tgt) ** 2))

    fd_tau = OA.fd_directional(L_tau, np.array([tau]), np.array([1.0]), rel=1e-3)
    assert gtau == pytest.approx(fd_tau, rel=RTOL_GRAD)


@pytest.mark.parametrize("scheme", ["euler", "heun", "ssprk3", "tsit5"])
@pytest.mark.parametrize("precision", ["fp32", "bf16x3"])
def test_step_vjp_fused_equals_torch_form(scheme, precision):
    """``qg_step_vjp`` (stage recomputation and reverse sweep in one C-ABI call with fused
    linear-combination kernels) against the same algebra written with torch operations around
    ``qg_rhs`` / ``qg_rhs_vjp``: the same kernels in the same order, so within FP32 rounding of
    the combination order (1e-6), for the state and the parameter cotangents.  Two calls in a
    row on the same workspace agree to the same bound (not bit for bit: the VJP stencil sums
    the layers' contributions to the modal right-hand side with atomic adds, whose order
    varies)."""
    from somax_gb300 import adjoint as A

    m, _ = pair(40, 33, 3, precision=precision, **PHYS)
    plan = m.plan()
    y0 = cuda(field(m.shape, 41)).reshape(-1)
    g = cuda(field(m.shape, 42, scale=1.0)).reshape(-1)
    pv = m._param_vector(y0.device)
    yb, pb = A.step_vjp(plan, y0, pv, 1200.0, scheme, g)
    yb2, pb2 = A.step_vjp(plan, y0, pv, 1200.0, scheme, g)
    yt, pt = A.step_vjp_torch(plan, y0, pv, 1200.0, scheme, g)
    assert plan.status() == 0
    assert rel(yb2, yb.cpu().double().numpy()) < 1e-6 and rel(pb2, pb.cpu().double().numpy()) < 1e-6
    assert rel(yb, yt.cpu().double().numpy()) < 1e-6
    for k in range(4):
        if float(pt[k]) != 0.0:
            assert abs(float(pb[k]) - float(pt[k])) <= 1e-5 * abs(float(pt[k])), (k, float(pb[k]), float(pt[k]))
