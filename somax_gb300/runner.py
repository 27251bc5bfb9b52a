"""Chunked integration with diagnostics between chunks: the runner's caller of the hot path.

Mirrors ``somax/_src/cli/_run.py``'s ``_chunked_integrate_with_diagnostics`` (:540-700) and its
helpers ``_build_diagnostic_grid`` (:504-537), ``_state_diagnostics`` (:408-432),
``_flatten_diagnostics`` (:138-167), ``_format_physical_scalars`` (:456-496) and
``IntegrationDivergedError`` (:38-45): the integration runs from one diagnostic time to the
next, logs per-field state statistics and the physical scalars of ``diagnose`` after every
chunk, warns when the energy grows tenfold between chunks and aborts on the first non-finite
state.  Any model of this package runs through it (``BaroclinicQG`` / ``BarotropicQG`` with
state ``q``; ``MultilayerShallowWater2D`` and ``ReparameterizedQG`` with state ``h, u, v``):
each chunk is one ``model.integrate`` call (graph-replayed or cluster-resident steps on the
GPU), the statistics of every state field are reduced on the device by one kernel
(``qg_state_stats`` / ``qg_swm_state_stats``: min / mean / max and the non-finite count, four
doubles read back per field), the divergence check also reads the kernels' device non-finite
flag, and the physical scalars come from the model's ``diagnose`` on the device.  With
``output_dir`` the run writes the reference's artifacts (``_run.py:346-364``):
``snapshots.zarr`` (every saved state, appended while the integration goes on: each state is
copied to pinned host memory on a side stream and written by a worker thread) and the restart
file ``final_state.zarr``; ``restart_state`` reads one back (``_run.py:840-862``).
"""

from __future__ import annotations

import concurrent.futures as cf
import dataclasses
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


def _fields(state) -> list:
    """(name, tensor) of every field of a state dataclass, in declaration order."""
    return [(f.name, getattr(state, f.name)) for f in dataclasses.fields(state)]


def _is_swm(model) -> bool:
    return hasattr(model, "swm") or type(model).__name__ == "MultilayerShallowWater2D"


def _swm_plan(model, device):
    return (model.swm if hasattr(model, "swm") else model).plan(device)


def state_diagnostics(state, model_or_plan) -> dict:
    """``_state_diagnostics``: per state field, min / mean / max over the finite entries and the
    count of non-finite entries, reduced on the device (``qg_state_stats`` through a QG model's
    plan, ``qg_swm_state_stats`` for the shallow-water states).  The second argument is the
    model, or the QG plan itself."""
    out = {}
    for name, x in _fields(state):
        x = x.detach().to(torch.float32).contiguous().reshape(-1)
        if hasattr(model_or_plan, "state_stats"):
            st = model_or_plan.state_stats(x)
        elif _is_swm(model_or_plan):
            st = _swm_plan(model_or_plan, x.device).field_stats(x)
        else:
            st = model_or_plan.plan(x.device).state_stats(x)
        mn, mean, mx, n_bad = (float(v) for v in st.cpu())
        out[name] = {"min": mn, "mean": mean, "max": mx, "nan": int(n_bad)}
    return out


def flatten_diagnostics(diag) -> dict:
    """``_flatten_diagnostics``: the 0-d fields of a diagnostics record as floats and per-layer
    vectors (up to 16 entries) as ``<field>_layer_<i>``; fields are left out (the reference
    summarises them into its metrics file, which this runner does not write)."""
    out = {}
    if diag is None or not dataclasses.is_dataclass(diag):
        return out
    for f in dataclasses.fields(diag):
        v = getattr(diag, f.name)
        if v is None:
            continue
        if isinstance(v, torch.Tensor):
            if v.dim() == 0:
                out[f.name] = float(v)
            elif v.dim() == 1 and v.numel() <= 16:
                for i, x in enumerate(v.tolist()):
                    out[f"{f.name}_layer_{i}"] = float(x)
        elif isinstance(v, np.ndarray) and v.ndim == 1 and v.size <= 16:
            for i, x in enumerate(v.tolist()):
                out[f"{f.name}_layer_{i}"] = float(x)
        elif isinstance(v, (int, float, np.floating)):
            out[f.name] = float(v)
    return out


_HEADLINE = ("total_energy", "total_kinetic_energy", "energy", "kinetic_energy", "total_enstrophy", "enstrophy")
_ENERGY = ("total_energy", "energy", "total_kinetic_energy", "kinetic_energy")


def physical_scalars(model, state) -> tuple:
    """``_format_physical_scalars``: (log line of the headline scalars, flattened record);
    never raises (a failing ``diagnose`` gives its message and an empty record)."""
    try:
        flat = flatten_diagnostics(model.diagnose(state))
    except Exception as exc:  # noqa: BLE001 - the reference logs and carries on
        return f"diagnose failed: {type(exc).__name__}: {exc}", {}
    parts = [f"{k}={flat[k]:.6e}" for k in _HEADLINE if k in flat]
    return " ".join(parts), flat


def _status(model, device) -> int:
    if _is_swm(model):
        return _swm_plan(model, device).status()
    return model.plan(device).status()


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

    def add(self, state, t: float) -> None:
        """Queue one state (a state dataclass, or the tensor of a one-field ``q`` state)."""
        fields = _fields(state) if dataclasses.is_dataclass(state) else [("q", state)]
        dev = fields[0][1].device
        hosts, done = {}, None
        if dev.type == "cuda":
            if self.stream is None:
                self.stream = torch.cuda.Stream(device=dev)
            ev = torch.cuda.Event()
            ev.record(torch.cuda.current_stream(dev))
            with torch.cuda.stream(self.stream):
                self.stream.wait_event(ev)
                for name, x in fields:
                    host = torch.empty(x.shape, dtype=x.dtype, pin_memory=True)
                    host.copy_(x, non_blocking=True)
                    x.record_stream(self.stream)
                    hosts[name] = host
            done = torch.cuda.Event()
            done.record(self.stream)
        else:
            hosts = {name: x.detach().clone() for name, x in fields}
        first, self.first = self.first, False

        def write():
            if done is not None:
                done.synchronize()
            st = self.state_cls(**{k: v[None] for k, v in hosts.items()})
            ds = qio.snapshots_to_dataset(st, np.array([t]), attrs=self.attrs)
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
    for name, x in _fields(st):
        if tuple(x.shape) != tuple(model.shape):
            raise ValueError(f"restart field {name} has shape {tuple(x.shape)}, the model expects "
                             f"{tuple(model.shape)}")
    return st


def _fmt_stats(d: dict) -> str:
    return " ".join(f"{k}[min={v['min']:.3e} mean={v['mean']:.3e} max={v['max']:.3e} nan={v['nan']}]"
                    for k, v in d.items())


def chunked_integrate_with_diagnostics(model, state0, save_ts, dt: float, *, diagnostics_per_save: int = 1,
                                       solver=None, log: Callable[[str], Any] | None = None,
                                       mode: str = "run", output_dir=None, attrs: dict | None = None):
    """Integrate ``state0`` through ``save_ts`` chunk by chunk with diagnostics in between.

    Returns a namespace with ``ys`` (the states at ``save_ts``, stacked: every field has a
    leading time axis) and ``diagnostics`` (one dict per chunk: ``t``, the per-field state
    statistics under ``stats``, and the flattened physical scalars, e.g. ``total_kinetic_energy``
    and ``total_enstrophy`` of the QG models or ``total_energy`` of the shallow-water ones).
    Raises ``IntegrationDivergedError`` at the first chunk whose state is not finite.  With
    ``output_dir``: ``snapshots.zarr`` (written while the run goes on; not for
    ``mode="spinup"``) and ``final_state.zarr``, both with ``attrs``; the namespace then also
    carries ``snapshots_path`` and ``final_state_path``."""
    log = log or logging.getLogger("somax_gb300.runner").debug
    diag_ts, save_indices = build_diagnostic_grid(save_ts, diagnostics_per_save)
    n_chunks = diag_ts.shape[0] - 1
    device = _fields(state0)[0][1].device
    line0, _ = physical_scalars(model, state0)
    log(f"chunk 0/{n_chunks} sim_t={diag_ts[0]:.1f} | {_fmt_stats(state_diagnostics(state0, model))}"
        + (f" | physics: {line0}" if line0 else "") + " | initial state")
    state, saved, records, prev_energy = state0, [state0], [], None
    out = Path(output_dir) if output_dir is not None else None
    writer = None
    if out is not None:
        out.mkdir(parents=True, exist_ok=True)
        if mode != "spinup":
            writer = SnapshotWriter(out / "snapshots.zarr", model.state_cls, attrs)
            writer.add(state0, float(diag_ts[0]))
    for i in range(n_chunks):
        t0, t1 = float(diag_ts[i]), float(diag_ts[i + 1])
        sol = model.integrate(state, t0, t1, dt, solver=solver)
        new_state = model.state_cls(**{name: x[-1] for name, x in _fields(sol.ys)})
        flag = _status(model, device)
        stats = state_diagnostics(new_state, model)
        bad = any(v["nan"] > 0 for v in stats.values()) or flag == _lib.K["QG_ERR_NONFINITE"]
        line, flat = ("", {}) if bad else physical_scalars(model, new_state)
        energy = next((flat[k] for k in _ENERGY if k in flat), None)
        warning = ""
        if prev_energy and energy is not None and np.isfinite(energy) and abs(energy) > 10 * abs(prev_energy):
            warning = f" !! energy grew {energy / prev_energy:.1f}x from previous chunk"
        if energy is not None and np.isfinite(energy):
            prev_energy = energy
        records.append(dict(flat, t=t1, stats=stats))
        log(f"chunk {i + 1}/{n_chunks} sim_t={t1:.1f} | {_fmt_stats(stats)}"
            + (f" | physics: {line}" if line else "") + warning)
        if bad:
            log(f"ABORT at chunk {i + 1}/{n_chunks}: non-finite state")
            if writer is not None:
                writer.close()
            raise IntegrationDivergedError(
                f"{mode} integration produced non-finite values during chunk {i + 1}/{n_chunks} "
                f"(sim_t={t1:.1f}); the values appeared between sim_t={t0:.1f} and sim_t={t1:.1f}.\n"
                f"  {_fmt_stats(stats)}")
        if (i + 1) in save_indices:
            saved.append(new_state)
            if writer is not None:
                writer.add(new_state, t1)
        state = new_state
    ys = model.state_cls(**{name: torch.stack([getattr(s, name) for s in saved]) for name, _ in _fields(state0)})
    res = SimpleNamespace(ys=ys, diagnostics=records, stats={})
    if out is not None:
        if writer is not None:
            writer.close()
            res.snapshots_path = out / "snapshots.zarr"
        res.final_state_path = out / "final_state.zarr"
        qio.save_state(state, res.final_state_path, time=float(diag_ts[-1]), attrs=attrs)
    return res
