"""Host logic of the benchmark and of the launch accounting, on CPU: the roofline of every
kernel class (the multi-launch classes, and the cluster engine's single launch) from
synthetic per-class timings, and the layer-per-warp sweep's strip classes that decide how
many kernels a step launches."""

import os
import sys
import types

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
from somax_gb300.qg import lsweep_classes  # noqa: E402


def workload(members):
    w = types.SimpleNamespace(members=members)
    w.cells = lambda: sum(nl * N * N for N, nl in members)
    w.gemm_flops_per_pass = lambda: sum(2.0 * nl * N ** 3 for N, nl in members)
    return w


def test_roofline_multi_launch_classes():
    W = workload([(130, 3)])
    lc = 3 * 130 * 130
    # class: (total ms, launches); the DST passes dominate
    stats = {0: (0.01, 1), 1: (8.0, 800), 2: (2.0, 200), 3: (0.01, 1), 4: (0.0, 0)}
    r = bench.roofline(W, stats, "bf16x3", "baroclinic3_128")
    assert r["kernel"] == "dst_gemm" and r["bound"] == "hbm"
    assert r["algorithmic_bytes_per_launch"] == 8.0 * lc
    assert r["avg_launch_us"] == pytest.approx(10.0)
    assert r["achieved"] == pytest.approx(8.0 * lc / 10e-6 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / bench.peaks()["hbm_gbs"])
    assert set(r["kernels"]) == {"prep", "dst_gemm", "rhs_stencil", "other"}


def test_roofline_cluster_engine_single_launch():
    """With the cluster engine only class 4 has timings: it is reported as the cluster
    kernel with the state in and out once per launch (8 B per layer-cell)."""
    W = workload([(66, 1)])
    stats = {k: (0.0, 0) for k in range(4)}
    stats[4] = (0.7, 1)
    r = bench.roofline(W, stats, "bf16x3", "barotropic_64", cluster=True)
    assert r["kernel"] == "cluster"
    assert r["algorithmic_bytes_per_launch"] == 8.0 * 66 * 66
    assert set(r["kernels"]) == {"cluster"}


class Spec(types.SimpleNamespace):
    pass


@pytest.mark.parametrize("nx,ny,rows,expected", [
    (128, 128, 16, {0, 1, 3, 4}),  # 130 wide: strips 0, 2 touch x edges, strip 1 only the top / bottom bands
    (64, 64, 16, {1, 3}),          # 66 wide: both strips touch the x edges
    (256, 256, 64, {0, 1, 3, 4}),
    (3, 5, 16, {1}),
    (128, 40, 32, {1, 4}),         # 42 rows: no band strictly inside (the 10-row remainder has its own band)
])
def test_lsweep_strip_classes(nx, ny, rows, expected):
    assert lsweep_classes(Spec(nx=nx, ny=ny, mask=None), rows) == expected


def test_lsweep_masked_member_is_its_own_class():
    assert lsweep_classes(Spec(nx=30, ny=30, mask=object()), 16) == {2}


def test_swm_workloads_and_launch_accounting():
    """The shallow-water bench workloads: the reference's swm_jet run (4320 Tsit5 steps of
    20 s = one model day per bench step) and the 1024^2 basin; their initial states (the jet of
    baroclinic_instability_swm; rest plus a 2 m anomaly); the gradient's launch count."""
    import numpy as np

    import somax_gb300 as sg
    from somax_gb300 import testcases as tc

    jet = tc.SWM_CONFIGS["swm_jet64"]
    assert jet.bench_steps * jet.dt == 86400.0 and jet.scheme == "tsit5" and jet.nl == 2
    y = tc.swm_initial_state(jet)
    m, s = sg.baroclinic_instability_swm(lateral_viscosity=1000.0, device="cpu")
    assert np.array_equal(y[1], s.u.numpy()) and np.array_equal(y[2], s.v.numpy())
    big = tc.swm_initial_state(tc.SWM_CONFIGS["swm3_1024"])
    assert big.shape == (3, 3, 1026, 1026) and big.dtype == np.float32
    anomaly = big[0] - np.asarray(tc.SWM3_1024.H, np.float32)[:, None, None]
    assert abs(float(np.abs(anomaly).max()) - 2.0) < 1e-3 and float(np.abs(big[1:]).max()) == 0.0
    assert np.array_equal(tc.swm_initial_state(tc.SWM3_1024, seed=0), big)
    # one Tsit5 step's adjoint: 5 stage + 5 combine launches, 6 cotangent initialisations,
    # 4 per stage (three VJP kernels and the y_bar update), 15 a_sm updates, the parameters
    assert bench.swm_grad_launches("cluster", 360, 30) == (1 + 12) + (360 - 12) + 360 * 56 + 1
    assert bench.swm_grad_launches("stages", 360, 30) == (1 + 360 * 6) + (360 - 12) * 6 + 360 * 56 + 1
