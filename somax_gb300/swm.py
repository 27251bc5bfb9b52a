"""``MultilayerShallowWater2D`` (``somax/_src/models/swm/multilayer.py``) on the GPU.

The right-hand side (``vector_field``, :150-200), the boundary rules
(``apply_boundary_conditions``, :202-219 and the wall helpers :366-410) and the constant-step
integration run in libqgcore.so (``qg_swm_*``, C ABI in include/qgcore.h): one fused kernel
computes dh, du, dv of every layer with the boundary rules applied as the state is read, and
a Butcher-form stepper combines the stages.  ``create`` keeps the reference's keyword
arguments (:259-363); ``diagnose`` (:221-257) reduces the energy and potential enstrophy from
the same C-grid operators on the device (torch, not a hot path).

The state is a ``MultilayerSW2DState`` (h, u, v, each (nl, Ny, Nx) with the ghost ring);
the library sees it packed as one (3, nl, Ny, Nx) float32 array.  Only the first-order upwind
mass flux (``method="upwind1"``, the reference's default) is implemented.  ``vector_field`` and
``integrate`` are differentiable in the state and the parameters (``swm_adjoint``: the
hand-written VJPs of the library, checkpointed recomputation through ``integrate``).
"""

from __future__ import annotations

import ctypes as C
import dataclasses

import numpy as np
import torch

from . import _lib
from .qg import SaveAt, Solution, SomaxModel, _solver_name, _stream_handle, check
from .reparameterized import MultilayerSW2DState
from .transforms import ModalTransform, StratificationProfile

K = _lib.K
_SCHEMES = {"euler": K["QG_SCHEME_EULER"], "heun": K["QG_SCHEME_HEUN"], "ssprk3": K["QG_SCHEME_SSPRK3"],
            "tsit5": K["QG_SCHEME_TSIT5"]}
_ENGINES = {"auto": K["QG_SWM_ENGINE_AUTO"], "stages": K["QG_SWM_ENGINE_STAGES"],
            "cluster": K["QG_SWM_ENGINE_CLUSTER"]}


@dataclasses.dataclass
class MultilayerSW2DParams:
    """Differentiable parameters (multilayer.py:43-55)."""

    lateral_viscosity: torch.Tensor
    bottom_drag: torch.Tensor
    wind_amplitude: torch.Tensor


@dataclasses.dataclass(frozen=True)
class MultilayerSW2DPhysConsts:
    """Frozen constants (multilayer.py:58-72)."""

    gravity: float = 9.81
    f0: float = 1e-4
    beta: float = 0.0
    n_layers: int = 2


@dataclasses.dataclass
class MultilayerSW2DDiagnostics:
    """Diagnostics (multilayer.py:75-95)."""

    energy: torch.Tensor
    total_energy: torch.Tensor
    enstrophy: torch.Tensor
    total_enstrophy: torch.Tensor
    potential_vorticity: torch.Tensor
    relative_vorticity: torch.Tensor
    kinetic_energy_field: torch.Tensor


@dataclasses.dataclass(frozen=True)
class SWGrid:
    nx: int
    ny: int
    Lx: float
    Ly: float

    @property
    def Nx(self):
        return self.nx + 2

    @property
    def Ny(self):
        return self.ny + 2

    @property
    def dx(self):
        return self.Lx / self.nx

    @property
    def dy(self):
        return self.Ly / self.ny


class SwmPlan:
    """Owns a ``qg_swm_plan`` (device constants and stage buffers) on one device."""

    def __init__(self, desc: "_lib.SwmDesc", device):
        L = _lib.lib()
        d = torch.device(device)
        if d.type == "cuda" and d.index is None:
            d = torch.device("cuda", torch.cuda.current_device())
        self.device = d
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            check(L.qg_swm_create(C.byref(desc), C.byref(h)), "qg_swm_create")
        self._h, self._L = h, L
        self.state_size = int(L.qg_swm_state_size(h))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._L.qg_swm_destroy(h)
            except Exception:  # pragma: no cover
                pass
            self._h = None

    def _check(self, t, name):
        if not isinstance(t, torch.Tensor) or t.device.type != "cuda" or t.dtype != torch.float32:
            raise TypeError(f"{name} must be a float32 CUDA tensor")
        if t.device != self.device:
            raise ValueError(f"{name} is on {t.device}, the plan on {self.device}")
        if not t.is_contiguous() or t.numel() != self.state_size:
            raise ValueError(f"{name} must be contiguous with {self.state_size} elements")

    def _params(self, params) -> torch.Tensor:
        """(nu, kappa, tau0) as the contiguous float32 tensor on the plan's device the library reads."""
        params = torch.as_tensor(params).detach().to(device=self.device, dtype=torch.float32).contiguous()
        if params.numel() != 3:
            raise ValueError("params must hold 3 values (nu, kappa, tau0)")
        return params

    def rhs(self, y: torch.Tensor, params: torch.Tensor, apply_bc: bool, out=None) -> torch.Tensor:
        self._check(y, "state")
        params = self._params(params)
        out = torch.empty_like(y) if out is None else out
        self._check(out, "out")
        check(self._L.qg_swm_rhs(self._h, C.c_void_p(y.data_ptr()), C.c_void_p(out.data_ptr()),
                                 C.c_void_p(params.data_ptr()), K["QG_RHS_APPLY_BC"] if apply_bc else 0,
                                 _stream_handle(y.device)), "qg_swm_rhs")
        return out

    def apply_bc(self, y: torch.Tensor) -> torch.Tensor:
        self._check(y, "state")
        check(self._L.qg_swm_apply_bc(self._h, C.c_void_p(y.data_ptr()), _stream_handle(y.device)), "qg_swm_apply_bc")
        return y

    def step(self, y: torch.Tensor, params: torch.Tensor, dt: float, n_steps: int, scheme: str, apply_bc: bool):
        self._check(y, "state")
        params = self._params(params)
        check(self._L.qg_swm_step(self._h, C.c_void_p(y.data_ptr()), C.c_void_p(params.data_ptr()), float(dt),
                                  int(n_steps), _SCHEMES[scheme], K["QG_STEP_APPLY_BC"] if apply_bc else 0,
                                  _stream_handle(y.device)), "qg_swm_step")
        return y

    def status(self) -> int:
        flags = C.c_int(0)
        return self._L.qg_swm_status(self._h, C.byref(flags), _stream_handle(self.device))

    def rhs_vjp(self, y: torch.Tensor, params: torch.Tensor, tend_bar: torch.Tensor, apply_bc: bool):
        """(state_bar, params_bar) = the VJP of ``rhs(y, params, apply_bc)`` for the cotangent
        ``tend_bar`` (``qg_swm_rhs_vjp``)."""
        self._check(y, "state")
        self._check(tend_bar, "tend_bar")
        params = self._params(params)
        out = torch.empty_like(y)
        pb = torch.empty(3, dtype=torch.float32, device=y.device)
        check(self._L.qg_swm_rhs_vjp(self._h, C.c_void_p(y.data_ptr()), C.c_void_p(params.data_ptr()),
                                     C.c_void_p(tend_bar.data_ptr()), C.c_void_p(out.data_ptr()),
                                     C.c_void_p(pb.data_ptr()), K["QG_RHS_APPLY_BC"] if apply_bc else 0,
                                     _stream_handle(y.device)), "qg_swm_rhs_vjp")
        return out, pb

    def bc_vjp(self, y_bar: torch.Tensor) -> torch.Tensor:
        """The transpose of ``apply_bc`` on a cotangent, in place (``qg_swm_bc_vjp``)."""
        self._check(y_bar, "state_bar")
        check(self._L.qg_swm_bc_vjp(self._h, C.c_void_p(y_bar.data_ptr()), _stream_handle(y_bar.device)),
              "qg_swm_bc_vjp")
        return y_bar

    def step_vjp(self, y0: torch.Tensor, params: torch.Tensor, dt: float, scheme: str, g: torch.Tensor):
        """(y0_bar, params_bar) of one step of ``scheme`` from ``y0`` for the cotangent ``g`` of its
        result (``qg_swm_step_vjp``; the workspace is kept per scheme)."""
        self._check(y0, "state")
        self._check(g, "cotangent")
        params = self._params(params)
        # the state and the cotangent are staged in fixed buffers (with the workspace, per
        # scheme), so that the library replays the step's captured adjoint graph every step
        bufs = getattr(self, "_vjp_bufs", {})
        self._vjp_bufs = bufs
        need = int(self._L.qg_swm_step_vjp_workspace(self._h, _SCHEMES[scheme]))
        b = bufs.get(scheme)
        if b is None or b[3].numel() < need or b[3].device != y0.device:
            b = (torch.empty_like(y0), torch.empty_like(y0), torch.empty(3, dtype=torch.float32, device=y0.device),
                 torch.empty(need, dtype=torch.float32, device=y0.device))
            bufs[scheme] = b
        yin, yb, pb, work = b
        yin.copy_(y0)
        yb.copy_(g)
        check(self._L.qg_swm_step_vjp(self._h, C.c_void_p(yin.data_ptr()), C.c_void_p(params.data_ptr()), float(dt),
                                      _SCHEMES[scheme], C.c_void_p(yb.data_ptr()), C.c_void_p(pb.data_ptr()),
                                      C.c_void_p(work.data_ptr()), _stream_handle(y0.device)),
              "qg_swm_step_vjp")
        return yb.clone(), pb.clone()

    def segment_vjp(self, y_start: torch.Tensor, params: torch.Tensor, dt: float, k: int, scheme: str,
                    g: torch.Tensor):
        """(y_start_bar, params_bar) of k steps of ``scheme`` from the checkpoint ``y_start`` for the
        cotangent ``g`` of the k-th state, in one call (``qg_swm_segment_vjp``: the segment's
        states recomputed and every step's adjoint in reverse, replayed as one graph while the
        staged buffers, dt, k and the scheme repeat)."""
        self._check(y_start, "state")
        self._check(g, "cotangent")
        params = self._params(params)
        bufs = getattr(self, "_seg_bufs", {})
        self._seg_bufs = bufs
        key = (scheme, int(k))
        need = int(self._L.qg_swm_segment_vjp_workspace(self._h, _SCHEMES[scheme], int(k)))
        b = bufs.get(key)
        if b is None or b[3].device != y_start.device:
            b = (torch.empty_like(y_start), torch.empty_like(y_start),
                 torch.empty(3, dtype=torch.float32, device=y_start.device),
                 torch.empty(need, dtype=torch.float32, device=y_start.device))
            bufs[key] = b
        yin, yb, pb, work = b
        yin.copy_(y_start)
        yb.copy_(g)
        check(self._L.qg_swm_segment_vjp(self._h, C.c_void_p(yin.data_ptr()), C.c_void_p(params.data_ptr()),
                                         float(dt), int(k), _SCHEMES[scheme], C.c_void_p(yb.data_ptr()),
                                         C.c_void_p(pb.data_ptr()), C.c_void_p(work.data_ptr()),
                                         _stream_handle(y_start.device)), "qg_swm_segment_vjp")
        return yb.clone(), pb.clone()

    def field_stats(self, x: torch.Tensor) -> torch.Tensor:
        """(min, mean, max) over the finite entries of the float32 CUDA tensor x and the count of
        its non-finite entries, as a float64 device tensor of 4 values (``qg_swm_state_stats``)."""
        if not isinstance(x, torch.Tensor) or x.device.type != "cuda" or x.dtype != torch.float32:
            raise TypeError("x must be a float32 CUDA tensor")
        if x.device != self.device:
            raise ValueError(f"x is on {x.device}, the plan on {self.device}")
        x = x.contiguous()
        out = torch.empty(4, device=x.device, dtype=torch.float64)
        check(self._L.qg_swm_state_stats(self._h, C.c_void_p(x.data_ptr()), int(x.numel()),
                                         C.c_void_p(out.data_ptr()), _stream_handle(x.device)), "qg_swm_state_stats")
        return out

    def set_engine(self, engine: str):
        """``"auto"`` (the cluster engine where the basin fits), ``"stages"`` (one launch per
        stage) or ``"cluster"`` (every step of a call in one thread-block cluster)."""
        check(self._L.qg_swm_set_engine(self._h, _ENGINES[engine]), "qg_swm_set_engine")

    def engine(self, scheme: str = "tsit5") -> dict:
        """The engine ``step`` uses for ``scheme``, the cluster's CTA count and the tuning times
        of 32 steps (ms; the fastest cluster size and the stage engine)."""
        c = C.c_int(0)
        t = (C.c_float * 2)()
        with torch.cuda.device(self.device):
            r = self._L.qg_swm_engine(self._h, _SCHEMES[scheme], C.byref(c), t)
        if r < 0:
            check(-r, "qg_swm_engine")
        return {"engine": "cluster" if r == K["QG_SWM_ENGINE_CLUSTER"] else "stages", "cluster_ctas": c.value,
                "tuning_ms": {"cluster": t[0], "stages": t[1]}}

    def set_profiling(self, on: bool):
        """CUDA events around every launch of ``step`` (graphs bypassed); resets the counters."""
        check(self._L.qg_swm_set_profiling(self._h, int(on)), "qg_swm_set_profiling")

    def kernel_stats(self, kclass: int):
        """(total ms, launches) of one kernel class (QG_SWM_K_RHS / QG_SWM_K_COMBINE) since
        profiling was switched on."""
        t, n = C.c_double(0.0), C.c_int64(0)
        check(self._L.qg_swm_kernel_stats(self._h, int(kclass), C.byref(t), C.byref(n)), "qg_swm_kernel_stats")
        return t.value, n.value


class MultilayerShallowWater2D(SomaxModel):
    """Multilayer 2D nonlinear shallow water model, vector-invariant form (multilayer.py:98-257)."""

    state_cls = MultilayerSW2DState

    def __init__(self, params, consts, grid, strat, modal, wind_profile, bc, method, engine="auto"):
        if engine not in _ENGINES:
            raise ValueError(f"engine must be one of {sorted(_ENGINES)}, got {engine!r}")
        self.engine = engine
        self.params = params
        self.consts = consts
        self.grid = grid
        self.strat = strat
        self.modal = modal
        self.wind_profile = wind_profile
        self.bc_type = bc
        self.method = method
        self._plans: dict = {}

    @staticmethod
    def create(nx: int = 64, ny: int = 64, Lx: float = 4e6, Ly: float = 4e6, g: float = 9.81,
               f0: float = 9.375e-5, beta: float = 1.754e-11, n_layers: int = 3,
               H=(400.0, 1100.0, 2600.0), g_prime=(9.81, 0.025, 0.0125), stratification=None,
               lateral_viscosity: float = 0.0, bottom_drag: float = 0.0, wind_amplitude: float = 0.0,
               wind_profile: str = "doublegyre", bc: str = "periodic", method: str = "upwind1",
               engine: str = "auto"):
        """``MultilayerShallowWater2D.create`` with the same keyword arguments, plus the stepping
        engine of ``step`` / ``integrate`` (``SwmPlan.set_engine``)."""
        if stratification is not None:
            strat = stratification
        else:
            if len(H) != n_layers or len(g_prime) != n_layers:
                raise ValueError(f"n_layers ({n_layers}), len(H) ({len(H)}), and len(g_prime) "
                                 f"({len(g_prime)}) must all be equal")
            strat = StratificationProfile.from_layers(H=list(H), g_prime=list(g_prime))
        if bc not in ("periodic", "wall"):
            raise ValueError(f"bc must be 'periodic' or 'wall', got {bc!r}")
        if method != "upwind1":
            raise ValueError(f"only the upwind1 mass flux is implemented, got {method!r}")
        modal = ModalTransform.from_stratification(strat, f0)
        params = MultilayerSW2DParams(*(torch.tensor(float(x)) for x in (lateral_viscosity, bottom_drag,
                                                                        wind_amplitude)))
        consts = MultilayerSW2DPhysConsts(gravity=g, f0=f0, beta=beta, n_layers=strat.nl)
        return MultilayerShallowWater2D(params, consts, SWGrid(nx, ny, Lx, Ly), strat, modal, wind_profile, bc,
                                        method, engine)

    # ---- plumbing -------------------------------------------------------------------------
    @property
    def shape(self):
        return (self.consts.n_layers, self.grid.Ny, self.grid.Nx)

    def _desc(self):
        d = _lib.SwmDesc()
        g = self.grid
        d.nx, d.ny, d.n_layers = g.nx, g.ny, self.consts.n_layers
        d.Lx, d.Ly, d.f0, d.beta = g.Lx, g.Ly, self.consts.f0, self.consts.beta
        for k in range(self.consts.n_layers):
            d.H[k] = float(self.strat.H[k])
            d.g_prime[k] = float(self.strat.g_prime[k])
        d.wind_profile = K["QG_WIND_SINGLE"] if self.wind_profile == "single" else K["QG_WIND_DOUBLEGYRE"]
        d.bc = K["QG_SWM_WALL"] if self.bc_type == "wall" else K["QG_SWM_PERIODIC"]
        return d

    def plan(self, device=None) -> SwmPlan:
        if not torch.cuda.is_available():
            raise RuntimeError("somax_gb300 needs a CUDA device (no CPU fallback)")
        dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        if dev.type != "cuda":
            dev = torch.device("cuda", torch.cuda.current_device())
        key = dev.index
        if key not in self._plans:
            self._plans[key] = SwmPlan(self._desc(), dev)
            self._plans[key].set_engine(self.engine)
        return self._plans[key]

    def _param_vector(self, device) -> torch.Tensor:
        p = self.params
        return torch.tensor([float(p.lateral_viscosity), float(p.bottom_drag), float(p.wind_amplitude)],
                            dtype=torch.float32, device=device)

    def _param_tensor(self, device) -> torch.Tensor:
        """(nu, kappa, tau0) as a float32 device tensor that keeps the parameters' autograd graph."""
        p = self.params
        vals = [v if isinstance(v, torch.Tensor) else torch.tensor(float(v))
                for v in (p.lateral_viscosity, p.bottom_drag, p.wind_amplitude)]
        return torch.stack([v.reshape(()).to(device=device, dtype=torch.float32) for v in vals])

    def _grad(self, *ts) -> bool:
        p = self.params
        vals = list(ts) + [p.lateral_viscosity, p.bottom_drag, p.wind_amplitude]
        return torch.is_grad_enabled() and any(isinstance(v, torch.Tensor) and v.requires_grad for v in vals)

    def pack(self, state) -> torch.Tensor:
        for name in ("h", "u", "v"):
            t = getattr(state, name)
            if tuple(t.shape) != self.shape:
                raise ValueError(f"{name} must have shape {self.shape}, got {tuple(t.shape)}")
        dev = state.h.device if state.h.device.type == "cuda" else torch.device("cuda", torch.cuda.current_device())
        return torch.stack([state.h, state.u, state.v]).to(device=dev, dtype=torch.float32).contiguous()

    def unpack(self, y: torch.Tensor) -> MultilayerSW2DState:
        y = y.view((3,) + self.shape)
        return MultilayerSW2DState(h=y[0], u=y[1], v=y[2])

    # ---- the model contract -------------------------------------------------------------
    def vector_field(self, t, state, args=None) -> MultilayerSW2DState:
        """Tendencies (dh, du, dv) of the state as given (multilayer.py:150-200)."""
        y = self.pack(state)
        plan = self.plan(y.device)
        if self._grad(state.h, state.u, state.v):
            from . import swm_adjoint

            return self.unpack(swm_adjoint.rhs(plan, y.reshape(-1), self._param_tensor(y.device), apply_bc=False))
        return self.unpack(plan.rhs(y.reshape(-1), self._param_vector(y.device), apply_bc=False))

    def apply_boundary_conditions(self, state) -> MultilayerSW2DState:
        """Periodic wrap or the wall rules (multilayer.py:202-219)."""
        y = self.pack(state).clone()
        self.plan(y.device).apply_bc(y.reshape(-1))
        return self.unpack(y)

    def step(self, state, dt: float, n_steps: int = 1, solver="tsit5", apply_bc: bool = True):
        """``n_steps`` constant steps on the GPU; BC on every stage input (and on the initial
        state with ``apply_bc``), the returned state as stepped."""
        y = self.pack(state).clone().reshape(-1)
        plan = self.plan(y.device)
        plan.step(y, self._param_vector(y.device), dt, n_steps, _solver_name(solver), apply_bc)
        return self.unpack(y)

    def integrate(self, state0, t0: float, t1: float, dt: float, solver=None, saveat=None, **kw) -> Solution:
        """``SomaxModel.integrate`` with constant steps (``core/model.py:53-88``; Tsit5 default)."""
        if kw.get("stepsize_controller") not in (None, "constant"):
            raise ValueError("only constant step sizes are supported")
        scheme = _solver_name(solver) if solver is not None else "tsit5"
        saveat = saveat or SaveAt(t1=True)
        n_total = int(round((t1 - t0) / dt))
        if abs(n_total * dt - (t1 - t0)) > 1e-9 * max(1.0, abs(t1 - t0)):
            raise ValueError("(t1 - t0) must be a whole number of steps")
        targets = [int(round((float(t) - t0) / dt)) for t in saveat.ts] if saveat.ts is not None else [n_total]
        if self._grad(state0.h, state0.u, state0.v):
            return self._integrate_grad(state0, t0, dt, targets, scheme, int(kw.get("checkpoint_every", 10)))
        y = self.pack(state0).clone().reshape(-1)
        plan = self.plan(y.device)
        pv = self._param_vector(y.device)
        plan.apply_bc(y)
        ys, done = [], 0
        for tgt in targets:
            if tgt < done:
                raise ValueError("saveat.ts must be increasing")
            if tgt > done:
                plan.step(y, pv, dt, tgt - done, scheme, False)
                done = tgt
            ys.append(y.clone().view((3,) + self.shape))
        st = torch.stack(ys)
        ts = torch.tensor([t0 + k * dt for k in targets], dtype=torch.float64)
        return Solution(ts=ts, ys=MultilayerSW2DState(h=st[:, 0], u=st[:, 1], v=st[:, 2]))

    def _integrate_grad(self, state0, t0, dt, targets, scheme, every) -> Solution:
        """``integrate`` through the checkpointed adjoint (``swm_adjoint.Integrate``): the saved
        states are differentiable in the initial state and the parameters."""
        from . import swm_adjoint

        y = self.pack(state0).reshape(-1)
        plan = self.plan(y.device)
        pv = self._param_tensor(y.device)
        ys, done, first = [], 0, True
        for tgt in targets:
            if tgt < done:
                raise ValueError("saveat.ts must be increasing")
            if tgt > done or first:
                y = swm_adjoint.integrate(plan, y, pv, dt, tgt - done, scheme, apply_bc=first, checkpoint_every=every)
                done, first = tgt, False
            ys.append(y.view((3,) + self.shape))
        st = torch.stack(ys)
        ts = torch.tensor([t0 + k * dt for k in targets], dtype=torch.float64)
        return Solution(ts=ts, ys=MultilayerSW2DState(h=st[:, 0], u=st[:, 1], v=st[:, 2]))

    def diagnose(self, state) -> MultilayerSW2DDiagnostics:
        """Energy (KE + g' h^2 / 2) and potential enstrophy (q^2 h_X / 2) per layer, PV and
        relative vorticity at X points, KE at T points (multilayer.py:221-257)."""
        y = self.pack(state).double()
        h, u, v = y[0], y[1], y[2]
        g = self.grid
        s = (slice(None), slice(1, -1), slice(1, -1))

        def interior(inner):
            out = torch.zeros_like(h)
            out[s] = inner
            return out

        ke = 0.5 * (interior(0.5 * (u[s] ** 2 + (u ** 2)[:, 1:-1, :-2])) +
                    interior(0.5 * (v[s] ** 2 + (v ** 2)[:, :-2, 1:-1])))
        zeta = interior((v[:, 1:-1, 2:] - v[s]) / g.dx - (u[:, 2:, 1:-1] - u[s]) / g.dy)
        yrow = torch.arange(g.Ny, dtype=torch.float64, device=h.device) * g.dy
        f = (self.consts.f0 + self.consts.beta * (yrow - g.Ly / 2.0))[:, None].expand(g.Ny, g.Nx)
        fX = 0.5 * (f[1:-1, 1:-1] + f[2:, 1:-1])
        hX = interior(0.25 * (h[s] + h[:, 1:-1, 2:] + h[:, 2:, 1:-1] + h[:, 2:, 2:]))
        q = torch.zeros_like(h)
        q[s] = (zeta[s] + fX) / hX[s]
        area = g.dx * g.dy
        gp = torch.tensor(np.asarray(self.strat.g_prime, float), dtype=torch.float64, device=h.device)
        energy = ke[s].sum(dim=(-2, -1)) * area + 0.5 * gp * (h[s] ** 2).sum(dim=(-2, -1)) * area
        ens = 0.5 * (q[s] ** 2 * hX[s]).sum(dim=(-2, -1)) * area
        return MultilayerSW2DDiagnostics(energy=energy, total_energy=energy.sum(), enstrophy=ens,
                                         total_enstrophy=ens.sum(), potential_vorticity=q.float(),
                                         relative_vorticity=zeta.float(), kinetic_energy_field=ke.float())

    def status(self) -> int:
        return self.plan().status()


__all__ = ["MultilayerShallowWater2D", "MultilayerSW2DParams", "MultilayerSW2DPhysConsts", "MultilayerSW2DDiagnostics",
           "MultilayerSW2DState", "NonlinearShallowWater2D", "NonlinearSW2DState", "NonlinearSW2DParams",
           "NonlinearSW2DPhysConsts", "NonlinearSW2DDiagnostics"]


# ---- the single-layer nonlinear model ---------------------------------------------------------
@dataclasses.dataclass
class NonlinearSW2DState:
    """``NonlinearSW2DState`` (``swm/nonlinear_2d.py:25-36``): h, u, v, each (Ny, Nx)."""

    h: torch.Tensor
    u: torch.Tensor
    v: torch.Tensor


@dataclasses.dataclass
class NonlinearSW2DParams:
    """Differentiable parameters (``nonlinear_2d.py:39-50``)."""

    lateral_viscosity: torch.Tensor
    bottom_drag: torch.Tensor
    wind_amplitude: torch.Tensor


@dataclasses.dataclass(frozen=True)
class NonlinearSW2DPhysConsts:
    """Frozen constants (``nonlinear_2d.py:53-66``)."""

    gravity: float = 9.81
    f0: float = 1e-4
    beta: float = 0.0
    H0: float = 100.0


@dataclasses.dataclass
class NonlinearSW2DDiagnostics:
    """Diagnostics (``nonlinear_2d.py:69-86``)."""

    energy: torch.Tensor
    enstrophy: torch.Tensor
    potential_vorticity: torch.Tensor
    relative_vorticity: torch.Tensor
    kinetic_energy_field: torch.Tensor


class NonlinearShallowWater2D(SomaxModel):
    """The single-layer nonlinear shallow-water model (``swm/nonlinear_2d.py:89-318``) on the
    multilayer engine: it is the one-layer case with g' = g and the wind stress applied to u
    without the division by the layer depth (the engine divides by H[0], which this model
    sets to 1; the mean depth H0 is a constant of the model, not of its right-hand side).
    States are (Ny, Nx) fields; every method converts to the one-layer packing and back."""

    state_cls = NonlinearSW2DState

    def __init__(self, swm: MultilayerShallowWater2D, consts: NonlinearSW2DPhysConsts):
        self.swm = swm
        self.consts = consts

    @staticmethod
    def create(nx: int = 64, ny: int = 64, Lx: float = 1e6, Ly: float = 1e6, g: float = 9.81, f0: float = 1e-4,
               beta: float = 0.0, H0: float = 100.0, lateral_viscosity: float = 0.0, bottom_drag: float = 0.0,
               wind_amplitude: float = 0.0, wind_profile: str = "doublegyre", bc: str = "periodic",
               method: str = "upwind1", engine: str = "auto") -> "NonlinearShallowWater2D":
        """``NonlinearShallowWater2D.create`` (``nonlinear_2d.py:236-318``) with the same keywords."""
        swm = MultilayerShallowWater2D.create(nx=nx, ny=ny, Lx=Lx, Ly=Ly, g=g, f0=f0, beta=beta, n_layers=1, H=(1.0,),
                                              g_prime=(g,), lateral_viscosity=lateral_viscosity,
                                              bottom_drag=bottom_drag, wind_amplitude=wind_amplitude,
                                              wind_profile=wind_profile, bc=bc, method=method, engine=engine)
        return NonlinearShallowWater2D(swm, NonlinearSW2DPhysConsts(gravity=g, f0=f0, beta=beta, H0=H0))

    @property
    def params(self):
        p = self.swm.params
        return NonlinearSW2DParams(p.lateral_viscosity, p.bottom_drag, p.wind_amplitude)

    @params.setter
    def params(self, value):
        self.swm.params = MultilayerSW2DParams(value.lateral_viscosity, value.bottom_drag, value.wind_amplitude)

    @property
    def grid(self):
        return self.swm.grid

    @property
    def shape(self):
        return (self.grid.Ny, self.grid.Nx)

    def plan(self, device=None) -> SwmPlan:
        return self.swm.plan(device)

    def _to3(self, state) -> MultilayerSW2DState:
        for name in ("h", "u", "v"):
            t = getattr(state, name)
            if tuple(t.shape) != self.shape:
                raise ValueError(f"{name} must have shape {self.shape}, got {tuple(t.shape)}")
        return MultilayerSW2DState(h=state.h[None], u=state.u[None], v=state.v[None])

    @staticmethod
    def _to2(state) -> NonlinearSW2DState:
        return NonlinearSW2DState(h=state.h[..., 0, :, :], u=state.u[..., 0, :, :], v=state.v[..., 0, :, :])

    def vector_field(self, t, state, args=None) -> NonlinearSW2DState:
        """Tendencies of the state as given (``nonlinear_2d.py:132-181``)."""
        return self._to2(self.swm.vector_field(t, self._to3(state), args))

    def apply_boundary_conditions(self, state) -> NonlinearSW2DState:
        """Periodic wrap or the wall rules (``nonlinear_2d.py:183-208``)."""
        return self._to2(self.swm.apply_boundary_conditions(self._to3(state)))

    def step(self, state, dt: float, n_steps: int = 1, solver="tsit5", apply_bc: bool = True) -> NonlinearSW2DState:
        return self._to2(self.swm.step(self._to3(state), dt, n_steps, solver, apply_bc))

    def integrate(self, state0, t0: float, t1: float, dt: float, solver=None, saveat=None, **kw) -> Solution:
        """``SomaxModel.integrate`` with constant steps (Tsit5 default); differentiable in the
        state and the parameters."""
        sol = self.swm.integrate(self._to3(state0), t0, t1, dt, solver=solver, saveat=saveat, **kw)
        return Solution(ts=sol.ts, ys=self._to2(sol.ys))

    def diagnose(self, state) -> NonlinearSW2DDiagnostics:
        """Energy (KE + g h^2 / 2) and potential enstrophy (q^2 h_X / 2) summed over the interior
        with the cell area, PV and relative vorticity at the X points, KE at the T points
        (``nonlinear_2d.py:209-233``)."""
        d = self.swm.diagnose(self._to3(state))
        return NonlinearSW2DDiagnostics(energy=d.total_energy, enstrophy=d.total_enstrophy,
                                        potential_vorticity=d.potential_vorticity[0],
                                        relative_vorticity=d.relative_vorticity[0],
                                        kinetic_energy_field=d.kinetic_energy_field[0])

    def status(self) -> int:
        return self.swm.status()
