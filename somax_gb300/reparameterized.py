"""The geostrophic projection of ``ReparameterizedQG`` (``somax/_src/models/qg/reparameterized.py``).

The reparameterized QG model is the multilayer shallow-water model plus the projection
P = G (Q G)^-1 Q onto the geostrophic manifold after every step (Thiry, Li, Memin & Roullet
2024).  This module mirrors the model's projection API (``create``, ``project``,
``_solve_helmholtz``, the geostrophic parts of ``diagnose``) on the same CUDA inversion as the
QG classes, through ``qg_project`` (C ABI): a PV kernel, the modal DST-I Helmholtz solve and a
reconstruction kernel.  The shallow-water right-hand side itself (``vector_field``) belongs to
the multilayer SWM, which this library does not carry.
"""

from __future__ import annotations

import ctypes as C
import dataclasses

import torch

from . import _lib
from .qg import MemberSpec, Plan, _stream_handle, check
from .transforms import ModalTransform, StratificationProfile


@dataclasses.dataclass
class MultilayerSW2DState:
    """``MultilayerSW2DState`` (``swm/multilayer.py``): layer thickness h and velocities u, v,
    each (nl, Ny, Nx) with the ghost ring (u on the east faces, v on the north faces)."""

    h: torch.Tensor
    u: torch.Tensor
    v: torch.Tensor


@dataclasses.dataclass
class ReparamQGGeostrophy:
    """The QG-specific fields of ``ReparamQGDiagnostics`` (``reparameterized.py:37-62``)."""

    psi: torch.Tensor
    u_ageostrophic: torch.Tensor
    v_ageostrophic: torch.Tensor


class ReparameterizedQG:
    """``ReparameterizedQG`` (``reparameterized.py:65-315``): the geostrophic projection."""

    def __init__(self, spec: MemberSpec, strat: StratificationProfile, modal: ModalTransform, precision="fp32",
                 refine=0):
        self.spec = spec
        self.strat = strat
        self.modal = modal
        self.precision = precision
        self.refine = refine
        self._plans: dict = {}

    @staticmethod
    def create(nx=64, ny=64, Lx=4e6, Ly=4e6, g=9.81, f0=9.375e-5, beta=1.754e-11, n_layers=3,
               H=(400.0, 1100.0, 2600.0), g_prime=(9.81, 0.025, 0.0125), stratification=None,
               lateral_viscosity=0.0, bottom_drag=0.0, wind_amplitude=0.0, wind_profile="doublegyre",
               bc="wall", method="upwind1", poisson_bc="dst", precision="fp32", refine=0,
               eigs="consistent") -> "ReparameterizedQG":
        """``ReparameterizedQG.create`` (``reparameterized.py:230-315``) with the same keyword
        arguments; the shallow-water ones (``g``, viscosity, drag, wind, ``method``) are
        accepted for the drop-in signature and do not enter the projection."""
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
        modal = ModalTransform.from_stratification(strat, f0, eigs)
        spec = MemberSpec(nx, ny, Lx, Ly, f0, beta, list(strat.H), list(strat.g_prime), False, wind_profile,
                          eigs, modal, None)
        return ReparameterizedQG(spec, strat, modal, precision, refine)

    @property
    def shape(self):
        return (self.spec.n_layers, self.spec.ny + 2, self.spec.nx + 2)

    def plan(self, device=None) -> Plan:
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

    def apply_boundary_conditions(self, state: MultilayerSW2DState) -> MultilayerSW2DState:
        """The projection step of ``apply_boundary_conditions`` (``reparameterized.py:186-189``);
        the wall BCs of the shallow-water state that precede it belong to the SWM."""
        return self.project(state)

    def _solve_helmholtz(self, q: torch.Tensor) -> torch.Tensor:
        """(Q G)^-1 (``reparameterized.py:125-140``): modal Helmholtz solve, zero ring."""
        q = self._field(q, "q")
        return self.plan(q.device).invert(q)

    def diagnose(self, state: MultilayerSW2DState) -> ReparamQGGeostrophy:
        """The QG fields of ``diagnose`` (``reparameterized.py:191-228``): psi and the
        ageostrophic velocity u - u_g, v - v_g (the SWM energies are the SWM's)."""
        _, ug, vg, psi = self._project(state)
        return ReparamQGGeostrophy(psi=psi, u_ageostrophic=state.u - ug, v_ageostrophic=state.v - vg)

    def vector_field(self, t, state, args=None):
        raise NotImplementedError("the multilayer shallow-water right-hand side is not part of this library; "
                                  "ReparameterizedQG here provides the geostrophic projection")
