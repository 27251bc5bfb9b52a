"""qg_invert_static, the PV inversion that allocates no device memory, against qg_invert
and the float64 oracle.

Some callers cannot call cudaMalloc when they invert: code running inside a framework's
compiled program or memory pool, or a loop that bans allocation.  For them
qg_invert_static stages its work in a fixed device array compiled into libqgcore.so instead
of a plan's cudaMalloc'd workspace.  Its result must match the plan-based qg_invert and the
float64 restatement of ``_invert_pv`` (``baroclinic.py:135-159``, ``barotropic.py:113-121``)
within the inversion tolerance on consecutive calls (the second call reuses the scratch the
first one left behind), up to the largest member the fixed array holds (three layers of
512 x 512), and members beyond the fixed limit must be refused up front.
"""

import ctypes as C

import numpy as np
import pytest
import torch

import somax_gb300 as sg
from oracle import qg as O
from somax_gb300 import _lib
from somax_gb300 import testcases as tc

pytestmark = pytest.mark.gpu

RTOL_INV = 2e-6  # the inversion tolerance of tests/test_gpu_parity.py


def _rel(a, b):
    a = a.double()
    b = b.double()
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


def _call_static(model, q):
    desc = _lib.MemberDesc()
    model.spec.fill(desc)
    out = torch.full_like(q, float("nan"))
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = _lib.lib().qg_invert_static(C.byref(desc), C.c_void_p(q.data_ptr()), C.c_void_p(out.data_ptr()), stream)
    torch.cuda.synchronize()
    assert rc == 0, _lib.strerror(rc)
    return out


def test_invert_static_matches_qg_invert_on_consecutive_calls():
    cases = [
        sg.BaroclinicQG.create(nx=128, ny=128, Lx=5.12e6, Ly=5.12e6),  # 3 layers, 130 x 130
        sg.BarotropicQG.create(nx=37, ny=21),                          # ring kept, odd sizes
        sg.BaroclinicQG.create(nx=30, ny=44, n_layers=2, H=(500.0, 4500.0), g_prime=(9.81, 0.025)),
    ]
    for k, m in enumerate(cases):
        n = max(m.grid.nx, m.grid.ny)
        nl = 1 if m.barotropic else m.spec.n_layers
        base = tc.kminus3_field(n, seed=10 + k, nl=nl)[:, : m.grid.Ny, : m.grid.Nx] * 1e-6
        for call in range(2):  # two calls in a row on the same scratch
            q = torch.tensor((1.0 + call) * base.reshape(m.shape), dtype=torch.float32, device="cuda")
            ref = m._invert_pv(q)
            got = _call_static(m, q)
            assert torch.isfinite(got).all()
            assert _rel(got, ref) < RTOL_INV


def _oracle_model(m):
    g = m.grid
    if m.barotropic:
        return O.barotropic_model(nx=g.nx, ny=g.ny, Lx=g.Lx, Ly=g.Ly, f0=m.spec.f0, beta=m.spec.beta)
    return O.baroclinic_model(nx=g.nx, ny=g.ny, Lx=g.Lx, Ly=g.Ly, f0=m.spec.f0, beta=m.spec.beta,
                              H=tuple(m.spec.H), g_prime=tuple(m.spec.g_prime))


@pytest.mark.parametrize("case", ["baroclinic3_130", "barotropic_37x21", "baroclinic3_514"])
def test_invert_static_matches_oracle(case):
    m = {"baroclinic3_130": lambda: sg.BaroclinicQG.create(nx=128, ny=128, Lx=5.12e6, Ly=5.12e6),
         "barotropic_37x21": lambda: sg.BarotropicQG.create(nx=37, ny=21),
         # the largest member the fixed scratch holds: 3 x 514 x round_up(514, 32) = 2^20 - 6168 floats
         "baroclinic3_514": lambda: sg.BaroclinicQG.create(nx=512, ny=512, Lx=5.12e6, Ly=5.12e6)}[case]()
    o = _oracle_model(m)
    n = max(m.grid.nx, m.grid.ny)
    nl = 1 if m.barotropic else m.spec.n_layers
    base = tc.kminus3_field(n, seed=20, nl=nl)[:, : m.grid.Ny, : m.grid.Nx].reshape(m.shape) * 1e-6
    for call in range(2):
        q = torch.tensor((1.0 + call) * base, dtype=torch.float32, device="cuda")
        ref = O.invert_pv(o, q.cpu().double().numpy())
        got = _call_static(m, q)
        assert torch.isfinite(got).all()
        assert _rel(got.cpu(), torch.from_numpy(ref)) < RTOL_INV


def test_invert_static_refuses_oversize_member():
    m = sg.BaroclinicQG.create(nx=600, ny=600)
    desc = _lib.MemberDesc()
    m.spec.fill(desc)
    q = torch.zeros(m.shape, device="cuda")
    rc = _lib.lib().qg_invert_static(C.byref(desc), C.c_void_p(q.data_ptr()), C.c_void_p(q.data_ptr()),
                                     C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == _lib.K["QG_ERR_TOO_LARGE"]
    assert "static scratch" in _lib.strerror(rc)
