"""Benchmark of the GB300 QG time step: member-days (model-days) per second.

Default workload (``--config ensemble256``): the 256-member ragged ensemble (96 one-layer 64^2,
96 three-layer 128^2, 48 three-layer 256^2 and 16 five-layer 256^2 double gyres) advanced
together by one plan with split-BF16x3 tensor-core DST passes.  One bench step = one model day
of every member (72 SSP-RK3 steps at dt = 1200 s).  ``--config baroclinic3_128`` runs the single
3-layer 128^2 basin instead.

  value      member-days/s with the state resident in HBM (CUDA events around each bench
             step, L2 flushed between steps), whole job over all ranks
  vs_baseline  value / the plain FP32 single-member path on the same members: every member
             advanced alone by its own FP32 plan (CUDA-core DST passes, no batching), one
             qg_step call per member and model day, timed in the same run
  e2e        the same metric through the public API with the state in pinned host memory:
             every bench step copies q host->device, integrates one day, copies q back
  roofline   achieved bandwidth / throughput of the dominant kernel class: each class's share
             of a profiled pass (CUDA events around every launch) applied to the timed step,
             against MEASURED_PEAKS.json; ``stencil_hbm`` is the stencil class's line
  cpu_baseline  the float32 NumPy/SciPy restatement of the reference's CPU path on a
             bounded sample of the same workload (rank 0, N = 1 only); the same leg checks
             parity: one member of each class after 10 steps against the float64 restatement

``--config swm_jet64`` (the reference's 2-layer 64^2 shallow-water jet run) and ``swm3_1024``
(a 3-layer 1024^2 shallow-water double gyre) time the multilayer shallow-water stepper
(``qg_swm_step``) instead, with their own roofline (k_swm_stage), CPU baseline
(the float32 restatement) and parity fields.

``--impl reference`` times that CPU restatement alone (the reference's JAX path cannot be
installed here) and prints the same line with ``"impl": "reference"``.

Multi-GPU runs (torchrun) are independent replicas: each rank integrates its own basin, no
data-path collective; timing is max over ranks.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

# the headline metric of the reference's benchmark configurations, for every workload here
METRIC = "QG model-days/sec per GB300 vs plain FP32 path at \u22641e-5 rel err; stencil HBM GB/s"
UNIT = "model-days/s"


def _env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


class Clocks:
    """Samples nvidia-smi SM clocks and throttle reasons while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.rows.append([c.strip() for c in out.split(",")])
            except Exception:
                return
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=6)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"], "src": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "src": "fallback"}


def masked_cpu_baseline(threads: int, min_seconds: float = 10.0):
    """The masked basin (3-layer 512^2, 15 % land) on the host: the float64 oracle with its
    cached sparse LU per mode (no capacitance step), whole SSP-RK3 steps until at least
    ``min_seconds``.  Returns (model-days/s, steps, seconds)."""
    from oracle import masked as OM
    from oracle import qg as O
    from somax_gb300 import testcases as tc

    O.set_workers(threads)
    cfg = tc.CONFIGS["baroclinic3_512"]
    kw = cfg.model_kwargs()
    om = O.baroclinic_model(nx=cfg.n, ny=cfg.n, Lx=cfg.L, Ly=cfg.L, f0=kw["f0"], beta=kw["beta"], H=cfg.H,
                            g_prime=cfg.g_prime, lateral_viscosity=cfg.lateral_viscosity,
                            bottom_drag=cfg.bottom_drag, wind_amplitude=kw["wind_amplitude"],
                            biharmonic_viscosity=cfg.biharmonic_viscosity)
    mask = tc.land_mask(cfg.n, cfg.n, frac=0.15, seed=0)
    q = tc.initial_pv(cfg, seed=0)
    q = OM.integrate(om, q, mask, cfg.dt, 1, cfg.scheme)  # warm (factorisations)
    steps, t0 = 0, time.perf_counter()
    while True:
        q = OM.integrate(om, q, mask, cfg.dt, 1, cfg.scheme)
        steps += 1
        el = time.perf_counter() - t0
        if el >= min_seconds:
            break
    return steps * cfg.dt / 86400.0 / el, steps, el


def cpu_baseline(cfg, threads: int, min_seconds: float = 10.0, chunk: int = 12):
    """Float32 oracle restatement of the RK step loop on the host cores: whole chunks of
    ``chunk`` steps until at least ``min_seconds`` have elapsed.  Returns (model-days/s,
    steps, seconds)."""
    from oracle import qg as O
    from somax_gb300 import testcases as tc

    O.set_workers(threads)
    kw = cfg.model_kwargs()
    om = O.baroclinic_model(nx=cfg.n, ny=cfg.n, Lx=cfg.L, Ly=cfg.L, f0=kw["f0"], beta=kw["beta"], H=cfg.H,
                            g_prime=cfg.g_prime, lateral_viscosity=cfg.lateral_viscosity,
                            bottom_drag=cfg.bottom_drag, wind_amplitude=kw["wind_amplitude"],
                            biharmonic_viscosity=cfg.biharmonic_viscosity)
    q = tc.initial_pv(cfg, seed=0).astype(np.float32)
    O.integrate(om, q, cfg.dt, 1, cfg.scheme)  # warm
    steps, t0 = 0, time.perf_counter()
    while True:
        q = O.integrate(om, q, cfg.dt, chunk, cfg.scheme).astype(np.float32)
        steps += chunk
        el = time.perf_counter() - t0
        if el >= min_seconds:
            break
    return steps * cfg.dt / 86400.0 / el, steps, el


def ensemble_cpu_rate(threads: int, min_seconds: float = 10.0):
    """member-days/s of the 256-member mix on the host: one member of each class timed for
    ``min_seconds / 4``; the ensemble's step time is the count-weighted sum."""
    from somax_gb300 import testcases as tc

    t_step, desc = 0.0, []
    for count, cfg in tc.C4_MIX:
        _, steps, el = cpu_baseline(cfg, threads, min_seconds / len(tc.C4_MIX), chunk=4)
        t_step += count * el / steps
        desc.append(f"{steps} steps of {cfg.name}")
    return 256 * tc.C4_MIX[0][1].dt / 86400.0 / t_step, ", ".join(desc)


ENSEMBLE_DESC = ("ensemble256: 96 x 1-layer 64^2 (Rd 50 km) + 96 x 3-layer 128^2 + 48 x 3-layer 256^2 + "
                 "16 x 5-layer 256^2 double gyres, tau0 ~ U(0.05, 0.12) N/m^2, ssprk3 dt=1200s")


def describe(name):
    """(metric, unit, workload text) of a bench configuration, shared by both arms."""
    from somax_gb300 import testcases as tc

    if name == "ensemble256":
        return METRIC, "member-days/s", ENSEMBLE_DESC + ", 72 steps = 1 model day per bench step"
    if name == "adjoint256":
        return (METRIC, UNIT,
                "adjoint256: one gradient per bench step of the quadratic misfit of the final layer-1 psi (seeded "
                "target) with respect to q0 and tau0 after 100 ssprk3 steps (dt=1200s) of the 3-layer 256x256 double "
                "gyre: forward with checkpoints every 10 steps, reverse sweep with segment recomputation and "
                "qg_step_vjp per step; value = model-days of forward + reverse integration per second "
                "(100 steps = 1.389 model days per gradient)")
    if name == "masked3_512":
        return (METRIC, UNIT,
                "masked3_512: 3-layer 512x512 double gyre (Lx=Ly=5120 km) with a seeded coastline (15 % of the "
                "T-cells land, ring land), one FP32 refinement sweep, FP64 capacitance correction, ssprk3 "
                "dt=1200s, 72 steps = 1 model day per bench step")
    cfg = tc.CONFIGS[name]
    steps = int(round(86400.0 / cfg.dt))
    return METRIC, UNIT, (f"{name}: {cfg.nl}-layer {cfg.n}x{cfg.n} double gyre (Lx=Ly=5120 km), "
                          f"{cfg.scheme} dt={cfg.dt:g}s, {steps} steps = 1 model day per bench step")


# ---- the multilayer shallow-water workloads ---------------------------------------------------
SWM_METRIC = "SWM model-days/sec per GB300; k_swm_stage / k_swm_cluster HBM GB/s"
SWM_DESC = {
    "swm_jet64": ("swm_jet64: the swm_jet run of the reference (baroclinic_instability_swm): 2-layer 64x64 periodic "
                  "multilayer shallow water, Lx=Ly=1000 km, H=(500,4500) m, g'=(9.81,0.025), nu=1000 m^2/s, "
                  "drag 1e-7/s, opposite 0.5 m/s jets; tsit5 dt=20s, 4320 steps = 1 model day per bench step"),
    "swm3_1024": ("swm3_1024: 3-layer 1024x1024 wall-bounded multilayer shallow-water double gyre, Lx=Ly=4000 km, "
                  "H=(400,1100,2600) m, nu=100 m^2/s, wind 8e-5 m^2/s^2, from rest + a seeded 2 m height anomaly; "
                  "tsit5 dt=10s, 360 steps = 1 model hour per bench step"),
}
SWM_STAGES = {"euler": 1, "heun": 2, "ssprk3": 3, "tsit5": 6}


def swm_cpu_rate(cfg, min_seconds: float = 10.0):
    """Model-days/s of the float32 restatement of the shallow-water step (oracle.swm: NumPy
    elementwise, one thread) on the host: whole steps until at least ``min_seconds``.
    Returns (model-days/s, steps, seconds)."""
    from oracle import qg as O
    from oracle import swm as W
    from somax_gb300 import testcases as tc

    o = W.create(**cfg.oracle_kwargs())
    y = np.stack(W.apply_boundary_conditions(o, *tc.swm_initial_state(cfg))).astype(np.float32)
    y = O.rk_step(lambda z: W.rhs(o, z), y, cfg.dt, cfg.scheme).astype(np.float32)  # warm
    steps, t0 = 0, time.perf_counter()
    while True:
        y = O.rk_step(lambda z: W.rhs(o, z), y, cfg.dt, cfg.scheme).astype(np.float32)
        steps += 1
        el = time.perf_counter() - t0
        if el >= min_seconds:
            break
    return steps * cfg.dt / 86400.0 / el, steps, el


def swm_parity(cfg, plan, pv, dev):
    """Relative L2 of h, u, v after a few steps (10 up to 256^2, else 2) from the bench's initial
    state against the float64 restatement, each bounded by max(1e-5, 4 x the error of the
    same restatement run in float32) as in the shallow-water tests."""
    import torch

    from oracle import swm as W
    from somax_gb300 import testcases as tc

    n_steps = 10 if cfg.n <= 256 else 2
    o = W.create(**cfg.oracle_kwargs())
    y0 = tc.swm_initial_state(cfg)
    y = torch.tensor(y0, device=dev).reshape(-1)
    plan.step(y, pv, cfg.dt, n_steps, cfg.scheme, True)
    if plan.status() != 0:
        raise RuntimeError("shallow-water parity run flagged a non-finite tendency")
    got = y.view(y0.shape).cpu().double().numpy()
    ref = W.integrate(o, y0.astype(np.float64), cfg.dt, n_steps, cfg.scheme)
    f32 = W.integrate(o, y0, cfg.dt, n_steps, cfg.scheme)

    def rel(a, b):
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

    out, ok = {}, True
    for k, name in enumerate("huv"):
        e, floor = rel(got[k], ref[k]), rel(f32[k].astype(np.float64), ref[k])
        bound = max(1e-5, 4.0 * floor)
        out[name] = {"rel_l2": e, "float32_restatement": floor, "bound": bound}
        ok &= e < bound
    return {"steps": n_steps, "fields": out, "pass": bool(ok),
            "against": "float64 NumPy restatement of multilayer.py:150-219 (interior-write C-grid operators)"}


def swm_roofline(cfg, plan, pv, dev, step_ms):
    """Achieved bandwidth of the stepping kernel from a profiled pass (CUDA events around every
    launch, graphs off) of min(bench steps, 64) steps, its time scaled to the timed bench step
    (the profiled pass's total against the timed time of as many steps).

    Algorithmic HBM bytes per layer-cell (lc = nl Ny Nx):
      k_swm_stage    stage s reads the step's state and s earlier stage derivatives (h, u, v:
                     12 B per state) and writes one state (its derivative, or the next state on
                     the last stage): (s + 2) x 12 B; a Tsit5 step runs s = 0..5, 324 B
      k_swm_cluster  the cluster engine (small basins): the state in and out once per launch,
                     24 B; every stage input and derivative stays in the cluster's shared
                     memory, so the kernel is bound by its SMs' latency and cluster barriers,
                     not by HBM"""
    import torch

    from somax_gb300 import _lib
    from somax_gb300 import testcases as tc

    pk = peaks()
    ns = SWM_STAGES[cfg.scheme]
    lc = cfg.nl * (cfg.n + 2) ** 2
    P = min(cfg.bench_steps, 64)
    y = torch.tensor(tc.swm_initial_state(cfg), device=dev).reshape(-1)
    plan.set_profiling(True)
    plan.step(y, pv, cfg.dt, P, cfg.scheme, True)
    torch.cuda.synchronize()
    stats = {"swm_stage": plan.kernel_stats(_lib.K["QG_SWM_K_STAGE"]),
             "swm_cluster": plan.kernel_stats(_lib.K["QG_SWM_K_CLUSTER"])}
    plan.set_profiling(False)
    bytes_step = {"swm_stage": 12.0 * lc * sum(s + 2 for s in range(ns))}
    prof_total = sum(ms for ms, _ in stats.values())
    timed_ms = step_ms * P / cfg.bench_steps  # the timed bench step's share for P steps
    scale = timed_ms / prof_total if prof_total > 0 else 1.0
    traffic = traffic_table().get(cfg.name, {})
    kernels = {}
    for name, (ms, n) in stats.items():
        if not n:
            continue
        ms_t = ms * scale
        # the cluster engine moves the state through HBM once in and once out per launch
        total = bytes_step[name] * P if name in bytes_step else 24.0 * lc * n
        per_launch = total / n
        gbs = total / (ms_t / 1000.0) / 1e9
        kernels[name] = {"launches": n, "total_ms": ms_t, "avg_us": ms_t * 1000.0 / n,
                         "bytes_per_launch": per_launch, "achieved_gbs": gbs, "hbm_frac": gbs / pk["hbm_gbs"],
                         "bound": "hbm", "traffic": traffic.get(name)}
    dom = max(kernels, key=lambda k: kernels[k]["total_ms"])
    d = kernels[dom]
    step_bytes = sum(bytes_step.values())
    return {"bound": "hbm", "achieved": d["achieved_gbs"], "peak": pk["hbm_gbs"], "unit": "GB/s",
            "frac": d["hbm_frac"], "kernel": dom, "traffic": d["traffic"], "peak_src": pk["src"],
            "algorithmic_bytes_per_launch": d["bytes_per_launch"], "avg_launch_us": d["avg_us"],
            "step_bytes": step_bytes, "step_gbs": step_bytes / (step_ms / cfg.bench_steps / 1000.0) / 1e9,
            "durations": (f"each class's share of a profiled pass of {P} steps (CUDA events around every launch) "
                          f"applied to the timed bench step: profiled {prof_total:.3f} ms, timed {timed_ms:.3f} ms "
                          f"for {P} steps"),
            "kernels": kernels}


def run_swm(args, dev, world, rank, local):
    """The shallow-water bench line: ``--config swm_jet64`` or ``swm3_1024``."""
    import torch

    import somax_gb300 as sg
    from somax_gb300 import testcases as tc

    cfg = tc.SWM_CONFIGS[args.config]
    m = sg.MultilayerShallowWater2D.create(**cfg.model_kwargs(), engine=args.swm_engine)
    plan = m.plan(dev)
    pv = m._param_vector(dev)
    y0 = tc.swm_initial_state(cfg, seed=rank)
    y = torch.tensor(y0, device=dev).reshape(-1)
    plan.apply_bc(y)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > 129 MB L2
    for _ in range(args.warmup):
        plan.step(y, pv, cfg.dt, cfg.bench_steps, cfg.scheme, False)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        for k in range(args.steps):
            flush.fill_(float(k))
            ev[k][0].record()
            plan.step(y, pv, cfg.dt, cfg.bench_steps, cfg.scheme, False)
            ev[k][1].record()
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    dev_ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in ev), world, dev)
    ms_per_step = dev_ms / args.steps
    days = cfg.bench_steps * cfg.dt / 86400.0
    value = world * args.steps * days / (dev_ms / 1000.0)
    status = plan.status()

    # e2e: the C-ABI step with the state in pinned host memory (H2D, the steps, D2H)
    yh = torch.tensor(y0).reshape(-1).pin_memory()
    out = torch.empty_like(yh).pin_memory()
    yd = torch.empty_like(y)

    def host_step():
        yd.copy_(yh, non_blocking=True)
        plan.step(yd, pv, cfg.dt, cfg.bench_steps, cfg.scheme, True)
        out.copy_(yd, non_blocking=True)
        torch.cuda.current_stream(dev).synchronize()

    host_step()
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        host_step()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world, dev)
    e2e_value = world * args.steps * days / e2e_s

    roof = swm_roofline(cfg, plan, pv, dev, ms_per_step)
    ns = SWM_STAGES[cfg.scheme]
    line = {
        "metric": SWM_METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": SWM_DESC[cfg.name], "l2": "flushed between timed steps (256 MB write)",
                   "engine": plan.engine(cfg.scheme),
                   "graphs": "8-step CUDA graphs replayed (stage engine); one launch per call (cluster engine)",
                   "status": status,
                   "replicas": "independent basins per rank" if world > 1 else "one device"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": yh.numel() * 4,
                "d2h_bytes_per_step": out.numel() * 4,
                "api": "qg_swm_step (MultilayerShallowWater2D's plan) on a pinned host state copied in and out"},
        "roofline": roof,
        "gpu_launches": (1 if plan.engine(cfg.scheme)["engine"] == "cluster" else ns * cfg.bench_steps) * args.steps,
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, n, el = swm_cpu_rate(cfg, 10.0)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": f"{n} {cfg.scheme} steps of {cfg.name}, float32 NumPy restatement "
                                          f"(elementwise, one thread; {el:.1f} s)"}
        line["parity"] = swm_parity(cfg, plan, pv, dev)
    if rank == 0:
        print(json.dumps(line), flush=True)


SWM_GRAD_DESC = ("swm_grad_jet64: one gradient per bench step of the misfit 0.5 |h(T) - h_target|^2 of the "
                 "reference's swm_jet basin (2-layer 64x64 periodic, nu=1000) after 360 tsit5 steps (dt=20s, 2 model "
                 "hours; seeded 0.5 m target anomaly) with respect to h0, nu, kappa and tau0: forward with checkpoints "
                 "every 30 steps, reverse sweep with segment recomputation and qg_swm_step_vjp per step; value = model-"
                 "days of forward + reverse integration per second")


def swm_grad_launches(engine: str, n_steps: int, every: int, ns: int = 6) -> int:
    """Kernel launches of one Tsit5 gradient: the forward (boundary rules, then a call per
    checkpoint segment), the backward's recomputation (a one-step call per step of a segment
    but its first), one qg_swm_step_vjp per step (ns - 1 stage and combine launches, ns
    cotangent initialisations, per stage the three VJP kernels and the y_bar update, one update
    per non-zero a_sm, the parameter write-out) and the final transposed boundary rules."""
    segs = -(-n_steps // every)
    per_call = 1 if engine == "cluster" else None
    fwd = 1 + (segs if per_call else n_steps * ns)
    recompute = (n_steps - segs) * (1 if per_call else ns)
    vjp = 2 * (ns - 1) + ns + 4 * ns + ns * (ns - 1) // 2 + 1
    return fwd + recompute + n_steps * vjp + 1


def run_swm_grad(args, dev, world, rank, local):
    """The shallow-water adjoint's bench line (``--config swm_grad_jet64``)."""
    import torch

    import somax_gb300 as sg
    from somax_gb300 import testcases as tc

    cfg = tc.SWM_JET64
    n_steps, every = 360, 30
    m = sg.MultilayerShallowWater2D.create(**cfg.model_kwargs(), engine=args.swm_engine)
    y0 = tc.swm_initial_state(cfg, seed=rank)
    rng = np.random.default_rng(100 + rank)
    target = torch.tensor(y0[0] + 0.5 * rng.standard_normal(y0[0].shape), dtype=torch.float64, device=dev)
    base = (float(cfg.lateral_viscosity), float(cfg.bottom_drag), float(cfg.wind_amplitude))

    def gradient(h0):
        m.params = sg.MultilayerSW2DParams(*(torch.tensor(x, requires_grad=True) for x in base))
        h = h0.detach().clone().requires_grad_(True)
        u = torch.tensor(y0[1], device=dev)
        v = torch.tensor(y0[2], device=dev)
        sol = m.integrate(sg.MultilayerSW2DState(h=h, u=u, v=v), 0.0, n_steps * cfg.dt, cfg.dt, checkpoint_every=every)
        loss = 0.5 * ((sol.ys.h[-1].double() - target) ** 2).sum()
        loss.backward()
        return h.grad, m.params.lateral_viscosity.grad

    h0 = torch.tensor(y0[0], device=dev)
    for _ in range(args.warmup):
        gradient(h0)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        for k in range(args.steps):
            ev[k][0].record()
            gradient(h0)
            ev[k][1].record()
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    dev_ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in ev), world, dev)
    days = n_steps * cfg.dt / 86400.0
    value = world * args.steps * days / (dev_ms / 1000.0)
    # e2e: h0 from pinned host memory, the gradient back to pinned host memory
    hh = torch.tensor(y0[0]).pin_memory()
    out = torch.empty_like(hh).pin_memory()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        g, _ = gradient(hh.to(dev, non_blocking=True))
        out.copy_(g, non_blocking=True)
        torch.cuda.current_stream(dev).synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world, dev)
    line = {
        "metric": SWM_METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": SWM_GRAD_DESC, "engine": m.plan(dev).engine(cfg.scheme)},
        "e2e": {"value": world * args.steps * days / e2e_s, "unit": UNIT, "h2d_bytes_per_step": hh.numel() * 4,
                "d2h_bytes_per_step": out.numel() * 4, "api": "MultilayerShallowWater2D.integrate + autograd"},
        "gpu_launches": args.steps * swm_grad_launches(m.plan(dev).engine(cfg.scheme)["engine"], n_steps, every),
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import swm as W

        v, n, el = swm_cpu_rate(cfg, 10.0)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": f"{n} tsit5 steps of swm_jet64 forward only (the float32 restatement has no "
                                          f"reverse mode; {el:.1f} s)"}
        # d/d nu of 0.5 sum u^2 after 10 steps against float64 central differences of the
        # restatement (u is what nu acts on; the h misfit's derivative in nu is a small
        # difference of terms that FP32 holds to ~1e-3 and is not a parity measure)
        n10 = 10

        def oloss(nu):
            o = W.create(**dict(cfg.oracle_kwargs(), lateral_viscosity=nu))
            z = W.integrate(o, y0.astype(np.float64), cfg.dt, n10, "tsit5")
            return 0.5 * (z[1] ** 2).sum()

        m.params = sg.MultilayerSW2DParams(*(torch.tensor(x, requires_grad=True) for x in base))
        sol = m.integrate(sg.MultilayerSW2DState(*(torch.tensor(y0[k], device=dev) for k in range(3))), 0.0,
                          n10 * cfg.dt, cfg.dt)
        (0.5 * (sol.ys.u[-1].double() ** 2).sum()).backward()
        hnu = base[0] * 1e-4
        fd = (oloss(base[0] + hnu) - oloss(base[0] - hnu)) / (2 * hnu)
        got = float(m.params.lateral_viscosity.grad)
        line["parity"] = {"d_half_sum_u2_d_nu_10_steps": got, "float64_difference": fd,
                          "rel": abs(got - fd) / abs(fd), "bound": 1e-3,
                          "against": "float64 central differences of the NumPy restatement"}
    if rank == 0:
        print(json.dumps(line), flush=True)


def max_over_ranks(x: float, world: int, device) -> float:
    """The largest of every rank's x: a multi-rank job takes as long as its slowest rank."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world: int, n_members: int, steps: int, seconds: float) -> float:
    """Member-days per second of the whole job: every rank advances its own replica of
    n_members members by one model day per bench step."""
    return world * n_members * steps / seconds


def run_reference(args):
    """The reference's CPU path (its JAX code cannot be installed here): the float32
    NumPy/SciPy restatement on every host core, each bench step a bounded time sample."""
    from somax_gb300 import testcases as tc

    rank = _env_int("RANK", 0)
    if rank != 0:
        return
    threads = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    if args.config in tc.SWM_CONFIGS or args.config == "swm_grad_jet64":
        cfg = tc.SWM_CONFIGS.get(args.config, tc.SWM_JET64)
        vals, samples = [], []
        for k in range(args.warmup + args.steps):
            v, n, el = swm_cpu_rate(cfg, 5.0 if k >= args.warmup else 1.0)
            if k >= args.warmup:
                vals.append(v)
                samples.append(f"{n} {cfg.scheme} steps of {cfg.name} ({el:.1f} s)")
        value = statistics.median(vals)
        sample = (f"per bench step >= 5 s of the float32 NumPy restatement (elementwise, one thread), e.g. "
                  f"{samples[0]}; the reference's JAX path is not installable")
        print(json.dumps({
            "impl": "reference", "metric": SWM_METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / value, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": SWM_GRAD_DESC if args.config == "swm_grad_jet64" else SWM_DESC[cfg.name],
                       "sample": sample},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}), flush=True)
        return
    metric, unit, workload = describe(args.config)
    per_step_s = 5.0
    vals, samples = [], []
    for k in range(args.warmup + args.steps):
        if args.config == "ensemble256":
            v, desc = ensemble_cpu_rate(threads, per_step_s if k >= args.warmup else 1.0)
        elif args.config == "masked3_512":
            v, n, el = masked_cpu_baseline(threads, per_step_s if k >= args.warmup else 1.0)
            desc = f"{n} ssprk3 steps of masked3_512 in float64 with cached sparse LU ({el:.1f} s)"
        elif args.config == "adjoint256":
            v, n, el = cpu_baseline(tc.C5, threads, per_step_s if k >= args.warmup else 1.0)
            desc = f"{n} ssprk3 steps of baroclinic3_256 forward only (no CPU reverse mode; {el:.1f} s)"
        else:
            cfg = tc.CONFIGS[args.config]
            v, n, el = cpu_baseline(cfg, threads, per_step_s if k >= args.warmup else 1.0)
            desc = f"{n} {cfg.scheme} steps of {cfg.name} ({el:.1f} s)"
        if k >= args.warmup:
            vals.append(v)
            samples.append(desc)
    value = statistics.median(vals)
    sample = (f"per bench step >= {per_step_s:g} s of the float32 NumPy/SciPy restatement "
              f"(scipy.fft workers={threads}), e.g. {samples[0]}; the reference's JAX path is not installable")
    line = {
        "impl": "reference", "metric": metric, "value": value, "unit": unit, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / value,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload, "sample": sample},
        "cpu_baseline": {"value": value, "unit": unit, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


class Workload:
    """One bench step = one model day of every member, on one device."""

    def __init__(self, name, precision, persistent, dev, seed, stencil=None, gemm_tile=None, cluster=None, groups=1):
        import torch

        import somax_gb300 as sg
        from somax_gb300 import testcases as tc

        self.name = name
        self.c4 = None
        if name == "ensemble256":
            cfgs, models, q0s = [], [], []
            self.c4 = tc.c4_members(seed)
            for cfg, tau0, pv_seed in self.c4:
                models.append(sg.BaroclinicQG.create(**tc.member_kwargs(cfg, tau0), precision=precision,
                                                     persistent=persistent, cluster=cluster))
                q0s.append(tc.initial_pv(cfg, seed=pv_seed).astype(np.float32))
                cfgs.append(cfg)
            self.ens = sg.QGEnsemble(models, precision=precision, persistent=persistent, device=dev, stencil=stencil,
                                     gemm_tile=gemm_tile, cluster=cluster, groups=groups)
            self.plan = self.ens.plan
            self.params = self.ens.params(dev)
            self.q0 = np.concatenate([q.reshape(-1) for q in q0s])
            self.members = [(c.n + 2, c.nl) for c in cfgs]
            self.dt, self.scheme = cfgs[0].dt, cfgs[0].scheme
            self.model = None
        elif name == "adjoint256":
            cfg = tc.C5
            kw = cfg.model_kwargs()
            self.cfg, self.kw = cfg, kw
            self.model = sg.BaroclinicQG.create(**kw, precision=precision, stencil=stencil, gemm_tile=gemm_tile)
            self.plan = self.model.plan(dev)
            self.params = self.model._param_vector(dev)
            self.q0 = tc.initial_pv(cfg, seed=seed).astype(np.float32)
            tgt = torch.tensor(tc.initial_pv(cfg, seed=seed + 1), dtype=torch.float32, device=dev)
            self.target = self.model._invert_pv(tgt)[0].detach().double()
            self.members = [(cfg.n + 2, cfg.nl)]
            self.dt, self.scheme = cfg.dt, cfg.scheme
            self.adj_steps = 100
            self.ens = None
        else:
            masked = name == "masked3_512"
            cfg = tc.CONFIGS["baroclinic3_512" if masked else name]
            mask = tc.land_mask(cfg.n, cfg.n, frac=0.15, seed=0) if masked else None
            self.model = sg.BaroclinicQG.create(**cfg.model_kwargs(), precision=precision, persistent=persistent,
                                                stencil=stencil, gemm_tile=gemm_tile, mask=mask,
                                                refine=1 if masked else 0, cluster=cluster)
            self.plan = self.model.plan(dev)
            self.params = self.model._param_vector(dev)
            q0 = tc.initial_pv(cfg, seed=seed)
            if masked:
                q0 = np.where(mask == 0, 0.0, q0)
            self.q0 = q0.astype(np.float32)
            self.members = [(cfg.n + 2, cfg.nl)]
            self.dt, self.scheme = cfg.dt, cfg.scheme
            self.ens = None
        self.metric, self.unit, self.describe = describe(name)
        self.n_members = len(self.members)
        self.steps_per_day = int(round(86400.0 / self.dt))
        self.q = torch.tensor(self.q0, device=dev).reshape(-1)
        if name == "adjoint256":
            # a bench step integrates 100 steps forward and back: its rate in model days
            self.days_per_step = self.adj_steps * self.dt / 86400.0

    def gradient(self, q0):
        """(d loss / d q0, d loss / d tau0) through the public API: integrate with autograd."""
        import torch

        import somax_gb300 as sg

        kw = self.kw
        m = self.model
        m.params = sg.QGParams(torch.tensor(kw["lateral_viscosity"]), torch.tensor(kw["bottom_drag"]),
                               torch.tensor(float(kw["wind_amplitude"]), requires_grad=True),
                               torch.tensor(kw["biharmonic_viscosity"]))
        q = q0.detach().view(m.shape).requires_grad_(True)
        sol = m.integrate(sg.BaroclinicQGState(q=q), 0.0, self.adj_steps * self.dt, self.dt, solver=self.scheme,
                          checkpoint_every=10)
        psi = m._invert_pv(sol.ys.q[-1])
        loss = 0.5 * ((psi[0].double() - self.target) ** 2).sum()
        loss.backward()
        return q.grad, m.params.wind_amplitude.grad

    def device_step(self):
        if self.name == "adjoint256":
            self.gradient(self.q)
            return
        self.plan.step(self.q, self.params, self.dt, self.steps_per_day, self.scheme)

    def host_step(self, qh, out):
        """The public API with host buffers: H2D, one model day (or one gradient), D2H."""
        import somax_gb300 as sg

        if self.name == "adjoint256":
            q = qh.to(device=self.q.device, non_blocking=True)
            gq, _ = self.gradient(q)
            out.copy_(gq.reshape(-1), non_blocking=True)
            return
        if self.ens is not None:
            self.ens.step_host(qh, out, self.dt, self.steps_per_day, self.scheme)
        else:
            self.model.step(sg.BaroclinicQGState(q=qh.view(self.model.shape)), self.dt, self.steps_per_day,
                            self.scheme, out=out.view(self.model.shape))

    def cells(self):
        return sum(nl * N * N for N, nl in self.members)

    def gemm_flops_per_pass(self):
        return sum(2.0 * nl * N ** 3 for N, nl in self.members)


KERNEL_CLASSES = {0: "prep", 1: "dst_gemm", 2: "rhs_stencil", 3: "other", 4: "persistent"}


def traffic_table():
    """DRAM bytes per launch measured by ncu (dram__bytes_read.sum + dram__bytes_write.sum),
    committed with the profiles: {workload: {kernel class: bytes}}."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return {}
    with open(p) as f:
        return json.load(f).get("bytes_per_launch", {})


def roofline(W, stats, precision, name, cluster=False, step_ms=None):
    """Roofline of every kernel class from the profiled pass's per-launch event times.

    The profiled pass runs one bench step with CUDA events around every launch (graphs and
    the sweep's parallel branches still on, but every launch bracketed), so its classes add
    up to more than the timed step.  With ``step_ms`` (the timed bench step) each class's
    time is its share of the profiled pass times ``step_ms``, and achieved = algorithmic
    bytes per launch / (that time / launches).

    Algorithmic HBM bytes per launch, per layer-cell of every member (lc = sum nl Ny Nx):
      dst_gemm     one DST-I pass: operand in (4 B: FP32, or BF16 hi + lo) + result out (4 B)
      rhs_stencil  step mode: q of the stage, psi_hat, y0 in (12 B); y_next and the next
                   stage's modal operand out (8 B)
      prep / other pack q (4 B in, 8 B out) / unpack (4 B in, 4 B out)
      cluster      the cluster-resident step kernel (class 4 when the plan steps with it): the
                   state in (4 B) and out (4 B) once per launch; everything else lives in shared
                   memory, so the kernel is bound by its SMs' FP32 work and barriers, not HBM
    Issued tensor flops of a DST-I pass: 2 N per element (three products for BF16x3).  A
    kernel is HBM-bound when its bytes / peak bandwidth exceed its flops / peak throughput.
    The dominant class (largest total time) is the headline."""
    pk = peaks()
    lc = W.cells()
    bytes_per = {0: 12.0 * lc, 1: 8.0 * lc, 2: 20.0 * lc, 3: 8.0 * lc}
    if cluster:
        bytes_per[4] = 8.0 * lc
    flops_per = {1: W.gemm_flops_per_pass() * (3.0 if precision == "bf16x3" else 1.0)}
    traffic = traffic_table().get(name, {})
    prof_total = sum(ms for ms, n in stats.values() if n)
    scale = step_ms / prof_total if step_ms and prof_total > 0 else 1.0
    kernels = {}
    for k, (ms, n) in stats.items():
        if not n or k not in bytes_per:
            continue
        ms = ms * scale
        avg_s = ms / 1000.0 / n
        gbs = bytes_per[k] / avg_s / 1e9
        ent = {"launches": n, "total_ms": ms, "avg_us": avg_s * 1e6, "bytes_per_launch": bytes_per[k],
               "achieved_gbs": gbs, "hbm_frac": gbs / pk["hbm_gbs"]}
        if k in flops_per:
            tf = flops_per[k] / avg_s / 1e12
            ent.update({"issued_tflops": tf, "tensor_frac": tf / pk["bf16_tflops"]})
            t_hbm = bytes_per[k] / (pk["hbm_gbs"] * 1e9)
            t_tc = flops_per[k] / (pk["bf16_tflops"] * 1e12)
            ent["bound"] = "tensor" if t_tc > t_hbm else "hbm"
        else:
            ent["bound"] = "hbm"
        ent["traffic"] = traffic.get(KERNEL_CLASSES[k])
        kernels[KERNEL_CLASSES[k]] = ent
    if cluster and "persistent" in kernels:
        kernels["cluster"] = kernels.pop("persistent")
        dom_name = "cluster"
    else:
        dom_name = KERNEL_CLASSES[max((k for k in (1, 2) if KERNEL_CLASSES[k] in kernels), key=lambda k: stats[k][0])]
    d = kernels[dom_name]
    if d["bound"] == "tensor":
        roof = {"bound": "tensor", "achieved": d["issued_tflops"], "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                "frac": d["tensor_frac"]}
    else:
        roof = {"bound": "hbm", "achieved": d["achieved_gbs"], "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": d["hbm_frac"]}
    roof.update({"kernel": dom_name, "traffic": d["traffic"], "peak_src": pk["src"],
                 "algorithmic_bytes_per_launch": d["bytes_per_launch"], "avg_launch_us": d["avg_us"],
                 "durations": ("each class's share of a profiled pass (CUDA events around every launch) "
                               f"applied to the timed bench step: profiled {prof_total:.3f} ms, timed "
                               f"{step_ms:.3f} ms per step" if step_ms else "profiled pass, unscaled"),
                 "kernels": kernels})
    return roof


def plain_fp32_rate(dev, mix, repeats: int = 3):
    """Member-days/s of the plain FP32 single-member path on a mix of (count, config).

    One member of each class gets its own FP32 plan (DST passes on the CUDA cores, no
    batching, the library's default engine choice for that member alone) and is advanced one
    model day per ``qg_step`` call, timed with CUDA events on the launch stream (median of
    ``repeats`` days after a warm day).  Looping the members one after another takes the
    count-weighted sum of those days.  Returns (member-days/s, per-class details)."""
    import torch

    import somax_gb300 as sg
    from somax_gb300 import testcases as tc

    per_class, t_day, total = {}, 0.0, 0
    for count, cfg in mix:
        m = sg.BaroclinicQG.create(**cfg.model_kwargs(), precision="fp32")
        plan = m.plan(dev)
        params = m._param_vector(dev)
        q0 = torch.tensor(tc.initial_pv(cfg, seed=0).astype(np.float32), device=dev).reshape(-1)
        steps = int(round(86400.0 / cfg.dt))
        q = q0.clone()
        plan.step(q, params, cfg.dt, steps, cfg.scheme)  # warm: graph capture
        ts = []
        for _ in range(repeats):
            q.copy_(q0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            plan.step(q, params, cfg.dt, steps, cfg.scheme)
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        if plan.status(dev) != 0:
            raise RuntimeError(f"plain FP32 path flagged a device error on {cfg.name}")
        ms = statistics.median(ts)
        per_class[cfg.name] = {"members": count, "ms_per_model_day": ms,
                               "engine": "cluster" if plan.engine()["cluster_ctas"] else "multi-launch",
                               "stencil": plan.tuning()["stencil"]}
        t_day += count * ms
        total += count
    return total * 1000.0 / t_day, per_class


def parity_10_steps(W, dev, threads):
    """Interior relative L2 of q after 10 steps against the float64 restatement (part of the
    CPU-baseline leg): one member of each class of the ensemble, or the single basin.  The
    GPU run starts from the bench's initial state on a copy, outside the timed region."""
    import torch

    from oracle import masked as OM
    from oracle import qg as O
    from somax_gb300 import testcases as tc

    n_steps = 10
    O.set_workers(threads)
    q = torch.tensor(W.q0, device=dev).reshape(-1)
    W.plan.step(q, W.params, W.dt, n_steps, W.scheme)
    if W.plan.status(dev) != 0:
        raise RuntimeError("parity run flagged a device error")
    if W.ens is not None:
        got = W.ens.unpack(q)
        picks, seen = [], set()
        for i, (cfg, tau0, _) in enumerate(W.c4):
            if cfg.name not in seen:
                seen.add(cfg.name)
                picks.append((i, cfg, tc.member_kwargs(cfg, tau0)))
        cases = [(f"member {i} ({cfg.name})", cfg, kw, got[i], W.q0[W.ens.offsets[i]:W.ens.offsets[i] + W.ens.sizes[i]],
                  None) for i, cfg, kw in picks]
    else:
        masked = W.name == "masked3_512"
        cfg = tc.C5 if W.name == "adjoint256" else tc.CONFIGS["baroclinic3_512" if masked else W.name]
        mask = tc.land_mask(cfg.n, cfg.n, frac=0.15, seed=0) if masked else None
        cases = [(W.name, cfg, cfg.model_kwargs(), q.view(W.model.shape), W.q0, mask)]
    out = {}
    for label, cfg, kw, g, q0, mask in cases:
        om = O.baroclinic_model(nx=cfg.n, ny=cfg.n, Lx=cfg.L, Ly=cfg.L, f0=kw["f0"], beta=kw["beta"], H=cfg.H,
                                g_prime=cfg.g_prime, lateral_viscosity=cfg.lateral_viscosity,
                                bottom_drag=cfg.bottom_drag, wind_amplitude=kw["wind_amplitude"],
                                biharmonic_viscosity=cfg.biharmonic_viscosity)
        q0 = np.asarray(q0, np.float64).reshape(g.shape)
        if mask is None:
            ref = O.integrate(om, q0, cfg.dt, n_steps, cfg.scheme)
        else:
            ref = OM.integrate(om, q0, mask, cfg.dt, n_steps, cfg.scheme)
        gg = g.cpu().double().numpy()
        sl = (Ellipsis, slice(1, -1), slice(1, -1))
        out[label] = float(np.linalg.norm(gg[sl] - ref[sl]) / np.linalg.norm(ref[sl]))
    return {"rel_l2_10_steps": out, "max": max(out.values()), "bound": 1e-5,
            "against": "float64 NumPy/SciPy restatement of the reference (interior cells)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="ensemble256",
                    help="ensemble256 (default) | baroclinic3_128 | barotropic_64 | baroclinic3_256 | "
                         "baroclinic3_512 | baroclinic3_1024 | masked3_512 | adjoint256 | swm_jet64 | swm3_1024 | "
                         "swm_grad_jet64")
    ap.add_argument("--precision", default="bf16x3", help="DST-I GEMM arithmetic: fp32 | tf32 | bf16x3")
    ap.add_argument("--persistent", type=int, default=0,
                    help="1: all steps of a call in one persistent cooperative launch (tensor-core precisions)")
    ap.add_argument("--gemm-tile", type=int, default=None,
                    help="force the tensor-core DST tile width (144 | 80 | 48 | 32 | 16); default: autotuned")
    ap.add_argument("--stencil", default=None,
                    help="force a stencil variant (tile32x8 | tile64x16 | sweep16 | sweep32 | sweep64 | lsweep16 | lsweep32 | lsweep64); "
                         "default: the autotuner's pick")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--groups", type=int, default=1,
                    help="ensemble only: split the members into this many plans stepped concurrently on their own streams")
    ap.add_argument("--swm-engine", default="auto", choices=["auto", "stages", "cluster"],
                    help="shallow-water configs: the cluster engine where the basin fits, one launch per stage, "
                         "or the cluster engine forced")
    ap.add_argument("--cluster", default="auto", choices=["auto", "on", "off"],
                    help="cluster-resident stepping of small members: autotuned, forced on, or off")
    args = ap.parse_args()

    from somax_gb300 import testcases as tc

    if args.impl == "reference":
        run_reference(args)
        return

    import torch
    import torch.distributed as dist

    world = _env_int("WORLD_SIZE", 1)
    rank = _env_int("RANK", 0)
    local = _env_int("LOCAL_RANK", 0)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)

    if args.config == "swm_grad_jet64":
        run_swm_grad(args, dev, world, rank, local)
        if world > 1:
            dist.destroy_process_group()
        return
    if args.config in tc.SWM_CONFIGS:
        run_swm(args, dev, world, rank, local)
        if world > 1:
            dist.destroy_process_group()
        return

    W = Workload(args.config, args.precision, bool(args.persistent), dev, rank, args.stencil, args.gemm_tile,
                 {"auto": None, "on": True, "off": False}[args.cluster], args.groups)
    plan = W.plan
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > 129 MB L2

    for _ in range(args.warmup):
        W.device_step()
    torch.cuda.synchronize()

    # ---- timed region: device-resident state ------------------------------------------
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        for k in range(args.steps):
            flush.fill_(float(k))  # evict L2 between timed steps (outside the events)
            ev[k][0].record()
            W.device_step()
            ev[k][1].record()
        torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    dev_ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in ev), world, dev)
    ms_per_step = dev_ms / args.steps
    days = getattr(W, "days_per_step", 1.0)  # model days per bench step and member
    value = whole_job_rate(world, W.n_members, args.steps, dev_ms / 1000.0) * days
    status = plan.status(dev)

    # ---- e2e: public API with pinned host buffers --------------------------------------
    qh = torch.tensor(W.q0).reshape(-1).pin_memory()
    out = torch.empty_like(qh).pin_memory()
    W.host_step(qh, out)  # warm
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        W.host_step(qh, out)
        torch.cuda.current_stream(dev).synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world, dev)
    e2e_value = whole_job_rate(world, W.n_members, args.steps, e2e_s) * days
    qbytes = qh.numel() * 4

    # ---- profiled pass: per-kernel-class event timing (multi-launch path) ----------------
    plan.set_profiling(True)
    W.device_step()
    torch.cuda.synchronize()
    stats = {k: plan.kernel_stats(k) for k in range(5)}
    plan.set_profiling(False)

    # ---- launches per bench step (graph / persistent replay counts every kernel) ---------
    if args.config == "adjoint256":
        launches_per_day = sum(n for _, n in stats.values())  # every launch of one gradient, counted
    else:
        launches_per_day = plan.launches_per_call(W.steps_per_day, W.scheme)
    roof = roofline(W, stats, args.precision, args.config, plan.engine()["cluster_ctas"] > 0, ms_per_step)

    # ---- the plain FP32 single-member path on the same members (the metric's baseline) ----
    vs_baseline, plain = None, None
    if args.config not in ("masked3_512", "adjoint256"):
        mix = tc.C4_MIX if W.ens is not None else ((1, tc.CONFIGS[args.config]),)
        plain_rate, plain_classes = plain_fp32_rate(dev, mix)
        plain_rate *= world  # every rank loops its own replica of the members
        vs_baseline = value / plain_rate
        plain = {"value": plain_rate, "unit": W.unit, "per_class": plain_classes,
                 "how": "each member advanced alone by its own FP32 plan (CUDA-core DST passes, no batching), "
                        f"one qg_step call per member and model day, looped over the {W.n_members} member(s)"}

    line = {
        "metric": W.metric, "value": value, "unit": W.unit, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": vs_baseline, "dtype": "f32", "data": "synthetic",
        "config": {"workload": W.describe,
                   "precision": args.precision, "persistent": bool(args.persistent), "groups": args.groups,
                   "l2": "flushed between timed steps (256 MB write)",
                   "replicas": "independent basins per rank" if world > 1 else "one device",
                   "tuning": dict(plan.tuning(), engine=plan.engine()), "status": status},
        "e2e": {"value": e2e_value, "unit": W.unit, "h2d_bytes_per_step": qbytes, "d2h_bytes_per_step": qbytes,
                "api": "BaroclinicQG.step / QGEnsemble.step_host with pinned host q -> qg_step"},
        "roofline": roof,
        "stencil_hbm": ({"achieved_gbs": roof["kernels"]["rhs_stencil"]["achieved_gbs"],
                         "peak_gbs": peaks()["hbm_gbs"], "frac": roof["kernels"]["rhs_stencil"]["hbm_frac"]}
                        if "rhs_stencil" in roof["kernels"] else None),
        "gpu_launches": launches_per_day * args.steps,
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = len(os.sched_getaffinity(0))
        if args.config == "masked3_512":
            v, n, el = masked_cpu_baseline(threads, 10.0)
            sample = f"{n} ssprk3 steps of masked3_512, float64 NumPy/SciPy restatement with cached sparse LU ({el:.1f} s)"
        elif args.config == "adjoint256":
            v, n, el = cpu_baseline(tc.C5, threads, 10.0)
            sample = (f"{n} ssprk3 steps of baroclinic3_256, float32 NumPy/SciPy restatement, forward only "
                      f"({el:.1f} s): the CPU restatement has no reverse mode, and a gradient costs at least one "
                      "forward, so this overstates the CPU's gradient rate")
        elif W.model is not None:
            cfg = tc.CONFIGS[args.config]
            v, n, el = cpu_baseline(cfg, threads, 10.0)
            sample = f"{n} {cfg.scheme} steps of {cfg.name}, float32 NumPy/SciPy restatement ({el:.1f} s)"
        else:
            v, desc = ensemble_cpu_rate(threads, 10.0)
            sample = f"one member per class, count-weighted: {desc}; float32 NumPy/SciPy restatement"
        line["cpu_baseline"] = {"value": v, "unit": W.unit, "cores": threads, "kind": "port", "sample": sample}
        line["parity"] = parity_10_steps(W, dev, threads)
    if plain is not None:
        line["plain_fp32"] = plain
        line["config"]["vs_baseline"] = ("value / plain_fp32.value: the same members on the plain FP32 "
                                         "single-member path, timed in this run")
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
