"""Benchmark of the GB300 QG time step: model-days per second.

One bench step = one model day of integration (86400 / dt time steps) of the 3-layer
128x128 double-gyre basin with SSP-RK3 at dt = 1200 s (72 steps), run through libqgcore.

  value      model-days/s with the state resident in HBM (CUDA events around each bench
             step, L2 flushed between steps), whole job over all ranks
  e2e        the same metric through the public API with the state in pinned host memory:
             every bench step copies q host->device, integrates one day, copies q back
  roofline   achieved bandwidth / throughput of the dominant kernel class from CUDA-event
             timing of every launch in a profiled pass, against MEASURED_PEAKS.json
  cpu_baseline  the float32 NumPy/SciPy restatement of the reference's CPU path on a
             bounded sample of the same workload (rank 0, N = 1 only)

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

METRIC = "QG model-days/sec per GB300 (3-layer 128^2 double gyre, SSP-RK3 dt=1200 s)"
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


def cpu_baseline(cfg, sample_steps: int, threads: int):
    """Float32 oracle restatement of one RK step loop on the host cores."""
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
    t0 = time.perf_counter()
    O.integrate(om, q, cfg.dt, sample_steps, cfg.scheme)
    el = time.perf_counter() - t0
    days_per_s = sample_steps * cfg.dt / 86400.0 / el
    return days_per_s, el


def run_reference(args, cfg):
    rank = _env_int("RANK", 0)
    if rank != 0:
        return
    threads = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    sample = max(1, min(args.ref_sample_steps, int(round(86400 / cfg.dt))))
    for _ in range(args.warmup):
        cpu_baseline(cfg, 1, threads)
    vals, tot = [], 0.0
    for _ in range(args.steps):
        v, el = cpu_baseline(cfg, sample, threads)
        vals.append(v)
        tot += el
    value = statistics.median(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / value,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{cfg.name}: 3-layer {cfg.n}x{cfg.n} double gyre, {cfg.scheme} dt={cfg.dt:g}s",
                   "sample": f"{sample} time steps per bench step, scaled to model-days/s"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{sample} {cfg.scheme} steps of {cfg.name} in float32 NumPy/SciPy "
                                   f"(scipy.fft workers={threads}); the reference's JAX path is not installable"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="baroclinic3_128")
    ap.add_argument("--precision", default="fp32")
    ap.add_argument("--persistent", type=int, default=1, help="tensor-core precisions: one launch per call")
    ap.add_argument("--ref-sample-steps", type=int, default=12)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()

    from somax_gb300 import testcases as tc

    cfg = tc.CONFIGS[args.config]
    if args.impl == "reference":
        run_reference(args, cfg)
        return

    import torch
    import torch.distributed as dist

    import somax_gb300 as sg

    world = _env_int("WORLD_SIZE", 1)
    rank = _env_int("RANK", 0)
    local = _env_int("LOCAL_RANK", 0)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)

    model = sg.BaroclinicQG.create(**cfg.model_kwargs(), precision=args.precision, persistent=bool(args.persistent))
    steps_per_day = int(round(86400.0 / cfg.dt))
    q0 = tc.initial_pv(cfg, seed=rank).astype(np.float32)
    q = torch.tensor(q0, device=dev)
    plan = model.plan(dev)
    pv = model._param_vector(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > 129 MB L2

    def device_step(qt):
        plan.step(qt, pv, cfg.dt, steps_per_day, cfg.scheme)

    for _ in range(args.warmup):
        device_step(q)
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
            device_step(q)
            ev[k][1].record()
        torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    dev_ms = sum(a.elapsed_time(b) for a, b in ev)
    t = torch.tensor([dev_ms], device=dev, dtype=torch.float64)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dev_ms = float(t.item())
    ms_per_step = dev_ms / args.steps
    value = world * args.steps / (dev_ms / 1000.0)
    status = plan.status(dev)

    # ---- e2e: public API with pinned host buffers --------------------------------------
    qh = torch.tensor(q0).pin_memory()
    out = torch.empty_like(qh).pin_memory()
    model.step(sg.BaroclinicQGState(q=qh), cfg.dt, steps_per_day, cfg.scheme, out=out)  # warm
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        model.step(sg.BaroclinicQGState(q=qh), cfg.dt, steps_per_day, cfg.scheme, out=out)
        torch.cuda.current_stream(dev).synchronize()
    e2e_s = time.perf_counter() - t0
    t = torch.tensor([e2e_s], device=dev, dtype=torch.float64)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    e2e_value = world * args.steps / float(t.item())
    qbytes = qh.numel() * 4

    # ---- profiled pass: per-kernel-class event timing -----------------------------------
    plan.set_profiling(True)
    device_step(q)
    torch.cuda.synchronize()
    stats = {k: plan.kernel_stats(k) for k in range(4)}
    plan.set_profiling(False)
    launches_per_day = sum(n for _, n in stats.values()) - stats[0][1]  # prep runs once per call
    kern = {0: "prep", 1: "dst_gemm", 2: "rhs_stencil", 3: "other"}
    dom = max(stats, key=lambda k: stats[k][0])
    N = cfg.n + 2
    nl = cfg.nl
    cells = nl * N * N
    pk = peaks()
    stages = {"heun": 2, "ssprk3": 3}[cfg.scheme]
    if dom == 1:  # GEMM: 2 M N K flops per pass, M = nl N, N = K = N
        flop = 2.0 * nl * N * N * N
        avg_s = stats[1][0] / 1000.0 / stats[1][1]
        achieved = flop / avg_s / 1e12
        roof = {"bound": "tensor", "kernel": "dst_gemm", "achieved": achieved, "peak": pk["bf16_tflops"],
                "unit": "TFLOP/s", "frac": achieved / pk["bf16_tflops"], "traffic": None,
                "peak_src": pk["src"], "note": "GEMM passes are latency-bound at 130^2 (L2-resident)"}
    else:
        # stencil in step mode: read y_s, psi_hat, y0 (stages > 0), write y_next and the
        # next-stage modal operand: (5 * stages - 1) / stages * 4 bytes per cell per layer
        bpc = 4.0 * (5 * stages - 1) / stages
        avg_s = stats[dom][0] / 1000.0 / stats[dom][1]
        achieved = bpc * cells / avg_s / 1e9
        roof = {"bound": "hbm", "kernel": kern[dom], "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / pk["hbm_gbs"], "traffic": None, "peak_src": pk["src"]}
    roof["kernel_ms"] = {kern[k]: {"total_ms": v[0], "launches": v[1]} for k, v in stats.items()}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{cfg.name}: {nl}-layer {cfg.n}x{cfg.n} double gyre (Lx=Ly=5120 km), "
                               f"{cfg.scheme} dt={cfg.dt:g}s, {steps_per_day} steps = 1 model day per bench step",
                   "precision": args.precision, "l2": "flushed between timed steps (256 MB write)",
                   "replicas": "independent basin per rank" if world > 1 else "single basin",
                   "status": status},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": qbytes, "d2h_bytes_per_step": qbytes,
                "api": "BaroclinicQG.step(state with pinned host q) -> qg_step"},
        "roofline": roof,
        "gpu_launches": launches_per_day * args.steps,
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = len(os.sched_getaffinity(0))
        sample = 6
        v, el = cpu_baseline(cfg, sample, threads)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"{sample} {cfg.scheme} steps of {cfg.name}, float32 NumPy/SciPy "
                                          f"restatement ({el:.2f} s)"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
