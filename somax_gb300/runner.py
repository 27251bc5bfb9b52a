"""Chunked integration with diagnostics between chunks: the runner's caller of the hot path.

Mirrors ``somax/_src/cli/_run.py``'s ``_chunked_integrate_with_diagnostics`` (:540-700) and its
helpers ``_build_diagnostic_grid`` (:504-537), ``_state_diagnostics`` (:408-432) and
``IntegrationDivergedError`` (:38-45): the integration runs from one diagnostic time to the
next, logs state statistics and physical scalars after every chunk, warns when the energy
grows tenfold between chunks and aborts on the first non-finite state.  Here each chunk is one
``model.integrate`` call (graph-replayed fused steps on the GPU), the state statistics are
reduced on the device by one kernel (``qg_state_stats``: min / mean / max and the non-finite
count, four doubles read back), the divergence check also reads the kernels' device
non-finite flag (``qg_status``), and the physical scalars come from the fused diagnostics
kernel.  With ``output_dir`` the run writes the reference's artifacts (``_run.py:346-364``):
``snapshots.zarr`` (every saved state, appended while the integration goes on: each state is
copied to pinned host memory on a side stream and written by a worker thread) and the restart
file ``final_state.zarr``; ``restart_state`` reads one back (``_run.py:840-862``).
"""

from __future__ import annotations

import concurrent.futures as cf
import logging
from pathlib import Path
from types import SimpleNamespace
from typing import Any, Callable

import numpy as np
import torch

from . import _lib
from . import io as qio


class IntegrationDivergedError(RuntimeError):
    """An integration produced non-finite values (``_run.py:38-45``)."""


def build_diagnostic_grid(save_ts, diagnostics_per_save: int):
    """``_build_diagnostic_grid``: every save time plus ``diagnostics_per_save - 1`` evenly spaced
    interior points per save interval.  Returns ``(diag_ts, save_indices)`` with
    ``save_ts == diag_ts[sorted(save_indices)]``."""
    save_ts = np.asarray(save_ts, dtype=np.float64)
    n = max(int(diagnostics_per_save), 1)
    if n == 1:
        return save_ts, set(range(save_ts.shape[0]))
    parts = [float(save_ts[0])]
    for i in range(save_ts.shape[0] - 1):
        parts.extend(float(x) for x in np.linspace(save_ts[i], save_ts[i + 1], n + 1)[1:])
    return np.asarray(parts), {i * n for i in range(save_ts.shape[0])}


def state_diagnostics(state, plan) -> dict:
    """``_state_diagnostics``: min / mean / max over the finite entries and the count of
    non-finite entries of ``state.q``, reduced on the device by ``plan`` (``qg_state_stats``)."""
    q = state.q.detach().reshape(-1)
    mn, mean, mx, n_bad = (float(x) for x in plan.state_stats(q).cpu())
    return {"q": {"min": mn, "mean": mean, "max": mx, "nan": int(n_bad)}}


class SnapshotWriter:
    """Appends saved states to a ``snapshots.zarr`` store without holding up the integration:
    each state is copied device-to-host into pinned memory on a side stream (after an event on
    the integration's stream) and a single worker thread waits for that copy and writes it, in
    submission order.  ``close`` waits for every write."""

    def __init__(self, path, state_cls, attrs: dict | None = None):
        self.path = Path(path)
        self.state_cls = state_cls
        self.attrs = attrs or {}
        self.pool = cf.ThreadPoolExecutor(max_workers=1)
        self.jobs = []
        self.first = True
        self.stream = None

    def add(self, q: torch.Tensor, t: float) -> None:
        if q.device.type == "cuda":
            if self.stream is None:
                self.stream = torch.cuda.Stream(device=q.device)
            ev = torch.cuda.Event()
            ev.record(torch.cuda.current_stream(q.device))
            host = torch.empty(q.shape, dtype=q.dtype, pin_memory=True)
            with torch.cuda.stream(self.stream):
                self.stream.wait_event(ev)
                host.copy_(q, non_blocking=True)
                q.record_stream(self.stream)
            done = torch.cuda.Event()
            done.record(self.stream)
        else:
            host, done = q.detach().clone(), None
        first, self.first = self.first, False

        def write():
            if done is not None:
                done.synchronize()
            ds = qio.snapshots_to_dataset(self.state_cls(q=host[None]), np.array([t]), attrs=self.attrs)
            if first:
                qio.save_dataset(ds, self.path, mode="w")
            else:
                qio.append_to_dataset(ds, self.path)

        self.jobs.append(self.pool.submit(write))

    def close(self) -> None:
        for j in self.jobs:
            j.result()
        self.pool.shutdown()


def restart_state(path, model, device=None):
    """The state of a ``final_state.zarr`` (or the last snapshot of a snapshots store) for
    ``model``, on ``device`` (``_run.py:840-862``: the stored class must be the model's)."""
    ds = qio.load_dataset(path)
    st = qio.dataset_to_state(ds, model.state_cls, device=device)
    if tuple(st.q.shape) != tuple(model.shape):
        raise ValueError(f"restart state has shape {tuple(st.q.shape)}, the model expects {tuple(model.shape)}")
    return st


def _fmt_stats(d: dict) -> str:
    return " ".join(f"{k}[min={v['min']:.3e} mean={v['mean']:.3e} max={v['max']:.3e} nan={v['nan']}]"
                    for k, v in d.items())


def chunked_integrate_with_diagnostics(model, state0, save_ts, dt: float, *, diagnostics_per_save: int = 1,
                                       solver=None, log: Callable[[str], Any] | None = None,
                                       mode: str = "run", output_dir=None, attrs: dict | None = None):
    """Integrate ``state0`` through ``save_ts`` chunk by chunk with diagnostics in between.

    Returns a namespace with ``ys`` (the states at ``save_ts``, stacked: ``ys.q`` has a leading
    time axis) and ``diagnostics`` (one dict per chunk: ``t``, state statistics, total kinetic
    energy and enstrophy).  Raises ``IntegrationDivergedError`` at the first chunk whose state
    is not finite.  With ``output_dir``: ``snapshots.zarr`` (written while the run goes on;
    not for ``mode="spinup"``) and ``final_state.zarr``, both with ``attrs``; the namespace
    then also carries ``snapshots_path`` and ``final_state_path``."""
    log = log or logging.getLogger("somax_gb300.runner").debug
    diag_ts, save_indices = build_diagnostic_grid(save_ts, diagnostics_per_save)
    n_chunks = diag_ts.shape[0] - 1
    plan = model.plan(state0.q.device)
    log(f"chunk 0/{n_chunks} sim_t={diag_ts[0]:.1f} | {_fmt_stats(state_diagnostics(state0, plan))} | initial state")
    state, saved, records, prev_energy = state0, [state0.q], [], None
    out = Path(output_dir) if output_dir is not None else None
    writer = None
    if out is not None:
        out.mkdir(parents=True, exist_ok=True)
        if mode != "spinup":
            writer = SnapshotWriter(out / "snapshots.zarr", model.state_cls, attrs)
            writer.add(state0.q, float(diag_ts[0]))
    for i in range(n_chunks):
        t0, t1 = float(diag_ts[i]), float(diag_ts[i + 1])
        sol = model.integrate(state, t0, t1, dt, solver=solver)
        new_state = model.state_cls(q=sol.ys.q[-1])
        flag = plan.status()
        stats = state_diagnostics(new_state, plan)
        bad = stats["q"]["nan"] > 0 or flag == _lib.K["QG_ERR_NONFINITE"]
        energy = ens = float("nan")
        if not bad:
            dg = model.diagnose(new_state)
            energy, ens = float(dg.total_kinetic_energy), float(dg.total_enstrophy)
        warning = ""
        if prev_energy and np.isfinite(energy) and abs(energy) > 10 * abs(prev_energy):
            warning = f" !! energy grew {energy / prev_energy:.1f}x from previous chunk"
        if np.isfinite(energy):
            prev_energy = energy
        records.append({"t": t1, "stats": stats, "total_kinetic_energy": energy, "total_enstrophy": ens})
        log(f"chunk {i + 1}/{n_chunks} sim_t={t1:.1f} | {_fmt_stats(stats)} | physics: "
            f"total_kinetic_energy={energy:.6e} total_enstrophy={ens:.6e}{warning}")
        if bad:
            log(f"ABORT at chunk {i + 1}/{n_chunks}: non-finite state")
            if writer is not None:
                writer.close()
            raise IntegrationDivergedError(
                f"{mode} integration produced non-finite values during chunk {i + 1}/{n_chunks} "
                f"(sim_t={t1:.1f}); the values appeared between sim_t={t0:.1f} and sim_t={t1:.1f}.\n"
                f"  {_fmt_stats(stats)}")
        if (i + 1) in save_indices:
            saved.append(new_state.q)
            if writer is not None:
                writer.add(new_state.q, t1)
        state = new_state
    res = SimpleNamespace(ys=model.state_cls(q=torch.stack(saved)), diagnostics=records, stats={})
    if out is not None:
        if writer is not None:
            writer.close()
            res.snapshots_path = out / "snapshots.zarr"
        res.final_state_path = out / "final_state.zarr"
        qio.save_state(model.state_cls(q=state.q), res.final_state_path, time=float(diag_ts[-1]), attrs=attrs)
    return res
