"""Chunked integration with diagnostics between chunks: the runner's caller of the hot path.

Mirrors ``somax/_src/cli/_run.py``'s ``_chunked_integrate_with_diagnostics`` (:540-700) and its
helpers ``_build_diagnostic_grid`` (:504-537), ``_state_diagnostics`` (:408-432) and
``IntegrationDivergedError`` (:38-45): the integration runs from one diagnostic time to the
next, logs state statistics and physical scalars after every chunk, warns when the energy
grows tenfold between chunks and aborts on the first non-finite state.  Here each chunk is one
``model.integrate`` call (graph-replayed fused steps on the GPU), the state statistics are
reduced on the device, the divergence check also reads the kernels' device non-finite flag
(``qg_status``) instead of scanning the state on the host, and the physical scalars come from
the fused diagnostics kernel.
"""

from __future__ import annotations

import logging
from types import SimpleNamespace
from typing import Any, Callable

import numpy as np
import torch

from . import _lib


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


def state_diagnostics(state) -> dict:
    """``_state_diagnostics``: min / mean / max over the finite entries and the count of
    non-finite entries of ``state.q``, reduced on the device."""
    q = state.q.detach()
    finite = torch.isfinite(q)
    n_bad = int((~finite).sum())
    if n_bad == q.numel():
        return {"q": {"min": float("nan"), "mean": float("nan"), "max": float("nan"), "nan": n_bad}}
    qf = q[finite] if n_bad else q.reshape(-1)
    stats = torch.stack([qf.min(), qf.mean(), qf.max()]).double().cpu().numpy()
    return {"q": {"min": float(stats[0]), "mean": float(stats[1]), "max": float(stats[2]), "nan": n_bad}}


def _fmt_stats(d: dict) -> str:
    return " ".join(f"{k}[min={v['min']:.3e} mean={v['mean']:.3e} max={v['max']:.3e} nan={v['nan']}]"
                    for k, v in d.items())


def chunked_integrate_with_diagnostics(model, state0, save_ts, dt: float, *, diagnostics_per_save: int = 1,
                                       solver=None, log: Callable[[str], Any] | None = None,
                                       mode: str = "run"):
    """Integrate ``state0`` through ``save_ts`` chunk by chunk with diagnostics in between.

    Returns a namespace with ``ys`` (the states at ``save_ts``, stacked: ``ys.q`` has a leading
    time axis) and ``diagnostics`` (one dict per chunk: ``t``, state statistics, total kinetic
    energy and enstrophy).  Raises ``IntegrationDivergedError`` at the first chunk whose state
    is not finite."""
    log = log or logging.getLogger("somax_gb300.runner").debug
    diag_ts, save_indices = build_diagnostic_grid(save_ts, diagnostics_per_save)
    n_chunks = diag_ts.shape[0] - 1
    log(f"chunk 0/{n_chunks} sim_t={diag_ts[0]:.1f} | {_fmt_stats(state_diagnostics(state0))} | initial state")
    state, saved, records, prev_energy = state0, [state0.q], [], None
    plan = model.plan(state0.q.device)
    for i in range(n_chunks):
        t0, t1 = float(diag_ts[i]), float(diag_ts[i + 1])
        sol = model.integrate(state, t0, t1, dt, solver=solver)
        new_state = model.state_cls(q=sol.ys.q[-1])
        flag = plan.status()
        stats = state_diagnostics(new_state)
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
            raise IntegrationDivergedError(
                f"{mode} integration produced non-finite values during chunk {i + 1}/{n_chunks} "
                f"(sim_t={t1:.1f}); the values appeared between sim_t={t0:.1f} and sim_t={t1:.1f}.\n"
                f"  {_fmt_stats(stats)}")
        if (i + 1) in save_indices:
            saved.append(new_state.q)
        state = new_state
    return SimpleNamespace(ys=model.state_cls(q=torch.stack(saved)), diagnostics=records, stats={})
