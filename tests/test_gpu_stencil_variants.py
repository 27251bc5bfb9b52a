"""Every stencil variant (tile 32x8 / 64x16 with TMA halo boxes, column sweep with 16-, 32- and
64-row strips) against the float64 oracle, forced through ``qg_options.stencil`` so that the
autotuner's pick does not decide what is tested.  FP32 GEMMs isolate the stencil; the
ensemble case mixes layer counts (the sweep launches once per layer count)."""

import numpy as np
import pytest
import torch

import somax_gb300 as sg
from oracle import qg as O
from somax_gb300 import testcases as tc

pytestmark = pytest.mark.gpu

RTOL_RHS = 2e-5
RTOL_STEP = 1e-5
VARIANTS = sg.Plan.STENCIL_VARIANTS


def rel(a, b):
    a = a.detach().cpu().double().numpy() if isinstance(a, torch.Tensor) else a
    b = b.detach().cpu().double().numpy() if isinstance(b, torch.Tensor) else b
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def pair(nx, ny, nl, seed):
    H = (400.0, 1100.0, 2600.0, 900.0, 1500.0, 700.0, 300.0, 2000.0)[:nl] if nl > 1 else (4000.0,)
    g = (9.81, 0.025, 0.0125, 0.01, 0.008, 0.006, 0.004, 0.003)[:nl] if nl > 1 else (0.0055,)
    kw = dict(lateral_viscosity=60.0, bottom_drag=1e-7, wind_amplitude=1e-10, biharmonic_viscosity=1e9)
    m = sg.BaroclinicQG.create(nx=nx, ny=ny, Lx=1.2e6, Ly=1e6, n_layers=nl, H=H, g_prime=g, **kw)
    o = O.baroclinic_model(nx=nx, ny=ny, Lx=1.2e6, Ly=1e6, H=H, g_prime=g, **kw)
    rng = np.random.default_rng(seed)
    q = tc.kminus3_field(max(nx, ny), seed, nl)[:, : ny + 2, : nx + 2] * 1e-6
    q = q + 1e-7 * rng.standard_normal(q.shape)  # a non-zero ring too
    return m, o, q


SHAPES = [(3, 5, 2), (17, 13, 3), (30, 30, 1), (61, 29, 3), (24, 24, 5), (40, 33, 8), (100, 70, 4)]


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("nx,ny,nl", SHAPES)
def test_variant_rhs_and_steps(variant, nx, ny, nl):
    m, o, q = pair(nx, ny, nl, 40 + nl)
    plan = sg.Plan([m.spec], "fp32", stencil=variant)
    assert plan.tuning()["stencil"] == variant
    pv = m._param_vector(torch.device("cuda"))
    qd = torch.tensor(q, dtype=torch.float32, device="cuda")
    for bc in (False, True):
        ref = O.vector_field(o, O.zero_boundaries(q) if bc else q)
        assert rel(plan.rhs(qd, pv, apply_bc=bc), ref) < RTOL_RHS
    for scheme in ("heun", "ssprk3"):
        got = plan.step(qd.clone(), pv, 1200.0, 3, scheme)
        assert plan.status() == 0
        assert rel(got, O.integrate(o, q, 1200.0, 3, scheme)) < RTOL_STEP


@pytest.mark.parametrize("variant", ["sweep16", "sweep32", "sweep64", "lsweep16", "lsweep32", "lsweep64"])
def test_sweep_ensemble_mixed_layers(variant):
    specs = [((30, 30), 1, 3), ((40, 33), 3, 4), ((24, 24), 5, 5), ((130, 66), 2, 6), ((17, 13), 3, 7)]
    ms, os, qs = [], [], []
    for (nx, ny), nl, seed in specs:
        m, o, q = pair(nx, ny, nl, seed)
        ms.append(m)
        os.append(o)
        qs.append(q)
    ens = sg.QGEnsemble(ms, precision="bf16x3", persistent=False, stencil=variant)
    packed = ens.pack([torch.tensor(q, dtype=torch.float32, device="cuda") for q in qs])
    for d, o, q in zip(ens.unpack(ens.rhs(packed)), os, qs):
        # split-BF16x3 inversion inside: each intermediate plane holds ~16 mantissa bits, and
        # the last one (physical x, spectral y) leaves white-in-x noise in psi that the
        # Jacobian amplifies by ~1/dx^2; on the 130 x 66 member (dx 0.6 dy) that is 1.2e-4
        assert rel(d, O.vector_field(o, q)) < 2e-4
    ens.step(packed, 1200.0, 3, "ssprk3")
    assert ens.plan.status() == 0
    for got, o, q in zip(ens.unpack(packed), os, qs):
        assert rel(got, O.integrate(o, q, 1200.0, 3, "ssprk3")) < RTOL_STEP


@pytest.mark.parametrize("variant", ["sweep32", "lsweep16", "lsweep32", "lsweep64"])
@pytest.mark.parametrize("nx,ny,nl", [(130, 98, 3), (190, 150, 3), (125, 140, 2), (200, 140, 5)])
def test_sweep_equals_tile_stencil(variant, nx, ny, nl):
    """The column sweeps against the tile stencil on the same inversion (FP32 GEMMs), which
    isolates the stencil: these basins have layer-per-warp strips whose columns and rows all
    lie strictly inside the member (its interior kernel) beside edge strips, for every strip
    height; 125 gives an odd width.  At these sizes the FP32 inversion's own error against
    float64 (~2e-5 in the RHS at 192 x 152) would hide stencil differences."""
    m, _, q = pair(nx, ny, nl, 9)
    pv = m._param_vector(torch.device("cuda"))
    qd = torch.tensor(q, dtype=torch.float32, device="cuda")
    pa = sg.Plan([m.spec], "fp32", stencil="tile32x8")
    pb = sg.Plan([m.spec], "fp32", stencil=variant)
    for bc in (False, True):
        assert rel(pb.rhs(qd, pv, apply_bc=bc), pa.rhs(qd, pv, apply_bc=bc)) < 1e-6
    for scheme in ("heun", "ssprk3"):
        a = pa.step(qd.clone(), pv, 1200.0, 5, scheme)
        b = pb.step(qd.clone(), pv, 1200.0, 5, scheme)
        assert pb.status() == 0
        assert rel(b, a) < 1e-6


@pytest.mark.parametrize("precision", ["bf16x3", "tf32"])
@pytest.mark.parametrize("tile", [144, 80, 48, 32, 16])
@pytest.mark.parametrize("nx,ny,nl", [(3, 5, 2), (64, 64, 1), (128, 128, 3), (200, 130, 2), (256, 256, 3), (300, 17, 4)])
def test_gemm_tile_widths(precision, tile, nx, ny, nl):
    """Every tensor-core output tile width (144, 80, 48, 32, 16 columns, last tile of a member
    cut to a multiple of 16) against the float64 inversion."""
    m, o, q = pair(nx, ny, nl, 50 + nl)
    plan = sg.Plan([m.spec], precision, gemm_tile=tile)
    assert plan.tuning()["gemm_tile_n"] == tile
    psi = plan.invert(torch.tensor(q, dtype=torch.float32, device="cuda"))
    assert rel(psi, O.invert_pv(o, q)) < (3e-5 if precision == "bf16x3" else 6e-3)


@pytest.mark.parametrize("scheme", ["euler", "tsit5"])
@pytest.mark.parametrize("variant", ["tile32x8", "sweep16", "lsweep16"])
@pytest.mark.parametrize("precision", ["fp32", "bf16x3"])
def test_butcher_schemes_fused(scheme, variant, precision):
    """Euler and Tsit5 fused into qg_step (stencil in rhs mode + stage combine) against the
    oracle's Butcher-form stepping."""
    for nx, ny, nl in [(30, 24, 3), (17, 13, 1), (64, 40, 5)]:
        m, o, q = pair(nx, ny, nl, 60 + nl)
        plan = sg.Plan([m.spec], precision, stencil=variant)
        pv = m._param_vector(torch.device("cuda"))
        got = plan.step(torch.tensor(q, dtype=torch.float32, device="cuda"), pv, 1200.0, 3, scheme)
        assert plan.status() == 0
        assert rel(got, O.integrate(o, q, 1200.0, 3, scheme)) < RTOL_STEP
