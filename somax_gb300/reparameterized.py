"""``ReparameterizedQG`` (``somax/_src/models/qg/reparameterized.py``) on the GPU.

The reparameterized QG model is the multilayer shallow-water model plus the projection
P = G (Q G)^-1 Q onto the geostrophic manifold, applied to every stage input by
``apply_boundary_conditions`` (Thiry, Li, Memin & Roullet 2024).  As in the reference the model
wraps a ``MultilayerShallowWater2D`` (wall boundaries) and delegates ``vector_field``, the
parameters, constants and grid to it.  The projection runs on the same CUDA inversion as the
QG classes through ``qg_project`` (C ABI): a PV kernel, the modal DST-I Helmholtz solve and a
reconstruction kernel; ``step`` / ``integrate`` run the whole stage loop in the library
(``qg_reparam_step``: combine, wall rules, projection, shallow-water right-hand side).
"""

from __future__ import annotations

import ctypes as C
import dataclasses

import torch

from . import _lib
from .qg import MemberSpec, Plan, SaveAt, Solution, _solver_name, _stream_handle, check
from .transforms import ModalTransform, StratificationProfile


@dataclasses.dataclass
class MultilayerSW2DState:
    """``MultilayerSW2DState`` (``swm/multilayer.py``): layer thickness h and velocities u, v,
    each (nl, Ny, Nx) with the ghost ring (u on the east faces, v on the north faces)."""

    h: torch.Tensor
    u: torch.Tensor
    v: torch.Tensor


@dataclasses.dataclass
class ReparamQGDiagnostics:
    """``ReparamQGDiagnostics`` (``reparameterized.py:37-62``): the shallow-water diagnostics
    plus psi and the ageostrophic velocity u - u_g, v - v_g."""

    energy: torch.Tensor
    total_energy: torch.Tensor
    enstrophy: torch.Tensor
    total_enstrophy: torch.Tensor
    potential_vorticity: torch.Tensor
    relative_vorticity: torch.Tensor
    kinetic_energy_field: torch.Tensor
    psi: torch.Tensor
    u_ageostrophic: torch.Tensor
    v_ageostrophic: torch.Tensor


class ReparameterizedQG:
    """``ReparameterizedQG`` (``reparameterized.py:65-315``): multilayer SWM + the geostrophic
    projection."""

    state_cls = MultilayerSW2DState

    def __init__(self, swm, spec: MemberSpec, strat: StratificationProfile, modal: ModalTransform,
                 precision="fp32", refine=0):
        self.swm = swm
        self.spec = spec
        self.strat = strat
        self.modal = modal
        self.precision = precision
        self.refine = refine
        self._plans: dict = {}

    # delegate properties (reparameterized.py:95-123)
    @property
    def params(self):
        return self.swm.params

    @params.setter
    def params(self, value):
        self.swm.params = value

    @property
    def consts(self):
        return self.swm.consts

    @property
    def grid(self):
        return self.swm.grid

    @property
    def helmholtz_lambdas(self):
        return self.modal.eigenvalues * self.spec.f0 ** 2

    @staticmethod
    def create(nx=64, ny=64, Lx=4e6, Ly=4e6, g=9.81, f0=9.375e-5, beta=1.754e-11, n_layers=3,
               H=(400.0, 1100.0, 2600.0), g_prime=(9.81, 0.025, 0.0125), stratification=None,
               lateral_viscosity=0.0, bottom_drag=0.0, wind_amplitude=0.0, wind_profile="doublegyre",
               bc="wall", method="upwind1", poisson_bc="dst", precision="fp32", refine=0,
               eigs="consistent") -> "ReparameterizedQG":
        """``ReparameterizedQG.create`` (``reparameterized.py:230-315``) with the same keyword
        arguments: the shallow-water model with wall boundaries, and the projection's modal
        Helmholtz inversion (DST-I GEMMs in ``precision``, ``refine`` FP32 refinement sweeps)."""
        from .swm import MultilayerShallowWater2D

        if bc != "wall":
            raise ValueError(f"ReparameterizedQG requires wall BCs (got bc={bc!r}). The geostrophic projection "
                             "uses Dirichlet Helmholtz inversion which is incompatible with periodic BCs.")
        if poisson_bc != "dst":
            raise ValueError("only the Dirichlet DST-I inversion (poisson_bc='dst') is implemented")
        if stratification is not None:
            strat = stratification
        else:
            if len(H) != n_layers or len(g_prime) != n_layers:
                raise ValueError(f"n_layers ({n_layers}), len(H) ({len(H)}), and len(g_prime) "
                                 f"({len(g_prime)}) must all be equal")
            strat = StratificationProfile.from_layers(H=list(H), g_prime=list(g_prime))
        swm = MultilayerShallowWater2D.create(nx=nx, ny=ny, Lx=Lx, Ly=Ly, g=g, f0=f0, beta=beta,
                                              n_layers=strat.nl, stratification=strat,
                                              lateral_viscosity=lateral_viscosity, bottom_drag=bottom_drag,
                                              wind_amplitude=wind_amplitude, wind_profile=wind_profile, bc="wall",
                                              method=method)
        modal = ModalTransform.from_stratification(strat, f0, eigs)
        spec = MemberSpec(nx, ny, Lx, Ly, f0, beta, list(strat.H), list(strat.g_prime), False, wind_profile,
                          eigs, modal, None)
        return ReparameterizedQG(swm, spec, strat, modal, precision, refine)

    @property
    def shape(self):
        return (self.spec.n_layers, self.spec.ny + 2, self.spec.nx + 2)

    def plan(self, device=None) -> Plan:
        """The inversion's plan on ``device`` (the projection's modal Helmholtz solve)."""
        device = torch.device(device if device is not None else "cuda")
        if device.index is None:
            device = torch.device("cuda", torch.cuda.current_device())
        if device.index not in self._plans:
            self._plans[device.index] = Plan([self.spec], self.precision, self.refine, True, device, False)
        return self._plans[device.index]

    def _field(self, x: torch.Tensor, name: str) -> torch.Tensor:
        if not isinstance(x, torch.Tensor) or not x.is_cuda:
            raise TypeError(f"{name} must be a CUDA tensor (no CPU fallback)")
        if tuple(x.shape) != self.shape:
            raise ValueError(f"{name} has shape {tuple(x.shape)}, expected {self.shape}")
        return x.detach().to(torch.float32).contiguous()

    def _project(self, state: MultilayerSW2DState):
        h = self._field(state.h, "h")
        u = self._field(state.u, "u")
        v = self._field(state.v, "v")
        plan = self.plan(h.device)
        hg, ug, vg, psi = (torch.empty_like(h) for _ in range(4))
        ptr = [C.c_void_p(t.data_ptr()) for t in (h, u, v, hg, ug, vg, psi)]
        check(plan._L.qg_project(plan._h, *ptr, _stream_handle(h.device)), "qg_project")
        return hg, ug, vg, psi

    def project(self, state: MultilayerSW2DState) -> MultilayerSW2DState:
        """P = G (Q G)^-1 Q (``reparameterized.py:142-178``): the geostrophically balanced state."""
        hg, ug, vg, _ = self._project(state)
        return MultilayerSW2DState(h=hg, u=ug, v=vg)

    def _solve_helmholtz(self, q: torch.Tensor) -> torch.Tensor:
        """(Q G)^-1 (``reparameterized.py:125-140``): modal Helmholtz solve, zero ring."""
        q = self._field(q, "q")
        return self.plan(q.device).invert(q)

    # ---- the model contract -------------------------------------------------------------
    def vector_field(self, t, state, args=None) -> MultilayerSW2DState:
        """The shallow-water tendencies (``reparameterized.py:180-184``)."""
        return self.swm.vector_field(t, state, args)

    def apply_boundary_conditions(self, state) -> MultilayerSW2DState:
        """The SWM wall rules, then the projection (``reparameterized.py:186-189``)."""
        return self.project(self.swm.apply_boundary_conditions(state))

    def _run(self, y: torch.Tensor, dt: float, n_steps: int, scheme: str, apply_bc: bool):
        from .swm import _SCHEMES

        sp = self.swm.plan(y.device)
        sp._check(y, "state")
        qp = self.plan(y.device)
        pv = self.swm._param_vector(y.device)
        check(sp._L.qg_reparam_step(sp._h, qp._h, C.c_void_p(y.data_ptr()), C.c_void_p(pv.data_ptr()), float(dt),
                                    int(n_steps), _SCHEMES[scheme], _lib.K["QG_STEP_APPLY_BC"] if apply_bc else 0,
                                    _stream_handle(y.device)), "qg_reparam_step")
        return y

    def step(self, state, dt: float, n_steps: int = 1, solver="tsit5", apply_bc: bool = True) -> MultilayerSW2DState:
        """``n_steps`` constant steps on the GPU: the projection and the wall rules on every stage
        input (and on the initial state with ``apply_bc``), the returned state as stepped."""
        y = self.swm.pack(state).clone().reshape(-1)
        self._run(y, dt, n_steps, _solver_name(solver), apply_bc)
        return self.swm.unpack(y)

    def _grad(self, *ts) -> bool:
        return self.swm._grad(*ts)

    def integrate(self, state0, t0: float, t1: float, dt: float, solver=None, saveat=None, **kw):
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
        y = self.swm.pack(state0).clone().reshape(-1)
        self._run(y, dt, 0, scheme, True)
        ys, done = [], 0
        for tgt in targets:
            if tgt < done:
                raise ValueError("saveat.ts must be increasing")
            if tgt > done:
                self._run(y, dt, tgt - done, scheme, False)
                done = tgt
            ys.append(y.clone().view((3,) + self.shape))
        st = torch.stack(ys)
        ts = torch.tensor([t0 + k * dt for k in targets], dtype=torch.float64)
        return Solution(ts=ts, ys=MultilayerSW2DState(h=st[:, 0], u=st[:, 1], v=st[:, 2]))

    def _integrate_grad(self, state0, t0, dt, targets, scheme, every) -> Solution:
        """``integrate`` through the checkpointed adjoint: ``qg_reparam_step_vjp`` per step,
        ``qg_reparam_bc_vjp`` for the boundary conditions applied to the initial state."""
        from . import swm_adjoint

        y = self.swm.pack(state0).reshape(-1)
        stepper = _ReparamStepper(self, y.device)
        pv = self.swm._param_tensor(y.device)
        ys, done, first = [], 0, True
        for tgt in targets:
            if tgt < done:
                raise ValueError("saveat.ts must be increasing")
            if tgt > done or first:
                y = swm_adjoint.integrate(stepper, y, pv, dt, tgt - done, scheme, apply_bc=first,
                                          checkpoint_every=every)
                done, first = tgt, False
            ys.append(y.view((3,) + self.shape))
        st = torch.stack(ys)
        ts = torch.tensor([t0 + k * dt for k in targets], dtype=torch.float64)
        return Solution(ts=ts, ys=MultilayerSW2DState(h=st[:, 0], u=st[:, 1], v=st[:, 2]))

    def diagnose(self, state: MultilayerSW2DState) -> ReparamQGDiagnostics:
        """``diagnose`` (``reparameterized.py:191-228``): the shallow-water energies and
        enstrophies, psi of the state's PV and the ageostrophic velocity u - u_g, v - v_g."""
        sd = self.swm.diagnose(state)
        _, ug, vg, psi = self._project(state)
        return ReparamQGDiagnostics(energy=sd.energy, total_energy=sd.total_energy, enstrophy=sd.enstrophy,
                                    total_enstrophy=sd.total_enstrophy, potential_vorticity=sd.potential_vorticity,
                                    relative_vorticity=sd.relative_vorticity,
                                    kinetic_energy_field=sd.kinetic_energy_field, psi=psi,
                                    u_ageostrophic=state.u - ug, v_ageostrophic=state.v - vg)

    def status(self) -> int:
        """The shallow-water plan's non-finite flag (QG_OK or QG_ERR_NONFINITE), cleared."""
        return self.swm.status()


class _ReparamStepper:
    """The stepping interface of ``swm_adjoint.Integrate`` (apply_bc, step, step_vjp, bc_vjp) for
    the reparameterised model: ``qg_reparam_step`` / ``qg_reparam_step_vjp`` /
    ``qg_reparam_bc_vjp`` on the model's shallow-water and inversion plans."""

    def __init__(self, model: ReparameterizedQG, device):
        self.sp = model.swm.plan(device)
        self.qp = model.plan(device)
        self.L = self.sp._L
        self.ws = {}

    def _h(self):
        return self.sp._h, self.qp._h

    def apply_bc(self, y):
        return self.step(y, torch.zeros(3, dtype=torch.float32, device=y.device), 1.0, 0, "tsit5", True)

    def step(self, y, p, dt, k, scheme, apply_bc):
        from .swm import _SCHEMES

        self.sp._check(y, "state")
        p = self.sp._params(p)
        sp, qp = self._h()
        check(self.L.qg_reparam_step(sp, qp, C.c_void_p(y.data_ptr()), C.c_void_p(p.data_ptr()), float(dt), int(k),
                                     _SCHEMES[scheme], _lib.K["QG_STEP_APPLY_BC"] if apply_bc else 0,
                                     _stream_handle(y.device)), "qg_reparam_step")
        return y

    def step_vjp(self, y0, p, dt, scheme, g):
        from .swm import _SCHEMES

        self.sp._check(y0, "state")
        self.sp._check(g, "cotangent")
        p = self.sp._params(p)
        sp, qp = self._h()
        need = int(self.L.qg_reparam_step_vjp_workspace(sp, _SCHEMES[scheme]))
        if scheme not in self.ws or self.ws[scheme].numel() < need:
            self.ws[scheme] = torch.empty(need, dtype=torch.float32, device=y0.device)
        yb = g.clone()
        pb = torch.empty(3, dtype=torch.float32, device=y0.device)
        check(self.L.qg_reparam_step_vjp(sp, qp, C.c_void_p(y0.data_ptr()), C.c_void_p(p.data_ptr()), float(dt),
                                         _SCHEMES[scheme], C.c_void_p(yb.data_ptr()), C.c_void_p(pb.data_ptr()),
                                         C.c_void_p(self.ws[scheme].data_ptr()), _stream_handle(y0.device)),
              "qg_reparam_step_vjp")
        return yb, pb

    def bc_vjp(self, g):
        self.sp._check(g, "cotangent")
        sp, qp = self._h()
        check(self.L.qg_reparam_bc_vjp(sp, qp, C.c_void_p(g.data_ptr()), _stream_handle(g.device)),
              "qg_reparam_bc_vjp")
        return g
