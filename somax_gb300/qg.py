"""Drop-in QG model classes whose hot path runs in libqgcore (hand-written sm_103a kernels).

Mirrors the public API of ``somax/_src/models/qg/baroclinic.py`` (``BaroclinicQG``),
``somax/_src/models/qg/barotropic.py`` (``BarotropicQG``) and the ``SomaxModel`` contract
(``somax/_src/core/model.py``): ``create``, ``vector_field``, ``apply_boundary_conditions``,
``integrate``, ``diagnose``, ``_invert_pv``; plus ``step`` for in-place stepping.  Arrays are
float32 CUDA tensors laid out as in the reference, ``(nl, Ny, Nx)`` (``(Ny, Nx)`` for the
barotropic model), ``Ny = ny + 2``, ``Nx = nx + 2``.
"""

from __future__ import annotations

import ctypes as C
import dataclasses
import math
from typing import Sequence

import numpy as np
import torch

from . import _lib, adjoint
from ._lib import K, MemberDesc, Options, check
from .transforms import ModalTransform, StratificationProfile

PRECISIONS = {"fp32": K["QG_DST_FP32"], "tf32": K["QG_DST_TF32"], "bf16x3": K["QG_DST_BF16X3"]}
SCHEMES = {"euler": K["QG_SCHEME_EULER"], "heun": K["QG_SCHEME_HEUN"], "ssprk3": K["QG_SCHEME_SSPRK3"],
           "tsit5": K["QG_SCHEME_TSIT5"]}


# ---------------------------------------------------------------------------------------
# Solver / SaveAt stand-ins for the diffrax objects integrate() accepts (core/model.py:75-88)
# ---------------------------------------------------------------------------------------
class _Solver:
    name = ""

    def __repr__(self):
        return f"{type(self).__name__}()"


class Euler(_Solver):
    name = "euler"


class Heun(_Solver):
    name = "heun"


class SSPRK3(_Solver):
    name = "ssprk3"


class Tsit5(_Solver):
    name = "tsit5"


@dataclasses.dataclass
class SaveAt:
    t1: bool = False
    ts: Sequence[float] | None = None


@dataclasses.dataclass
class Solution:
    ts: torch.Tensor
    ys: object


def _solver_name(s) -> str:
    if s is None:
        return "tsit5"
    if isinstance(s, str):
        if s not in SCHEMES:
            raise ValueError(f"unknown solver {s!r}")
        return s
    if isinstance(s, _Solver):
        return s.name
    raise TypeError(f"unsupported solver {s!r}")


# ---------------------------------------------------------------------------------------
# State / params / diagnostics (core/types.py; baroclinic.py:23-88)
# ---------------------------------------------------------------------------------------
@dataclasses.dataclass
class State:
    q: torch.Tensor


class BaroclinicQGState(State):
    pass


class BarotropicQGState(State):
    pass


@dataclasses.dataclass
class QGParams:
    """Differentiable parameters (``baroclinic.py:37-48``) plus the biharmonic extension."""

    lateral_viscosity: torch.Tensor
    bottom_drag: torch.Tensor
    wind_amplitude: torch.Tensor
    biharmonic_viscosity: torch.Tensor

    def vector(self, device) -> torch.Tensor:
        vals = (self.lateral_viscosity, self.bottom_drag, self.wind_amplitude, self.biharmonic_viscosity)
        if any(isinstance(v, torch.Tensor) and v.requires_grad for v in vals):
            # keep the autograd connection to the parameters
            return torch.stack([torch.as_tensor(v, dtype=torch.float32, device=device).reshape(()) for v in vals])
        return torch.tensor([float(v) for v in vals], dtype=torch.float32).to(device)  # one copy


BaroclinicQGParams = QGParams
BarotropicQGParams = QGParams


@dataclasses.dataclass
class QGDiagnostics:
    psi: torch.Tensor
    u: torch.Tensor
    v: torch.Tensor
    kinetic_energy: torch.Tensor
    total_kinetic_energy: torch.Tensor
    enstrophy: torch.Tensor
    total_enstrophy: torch.Tensor
    relative_vorticity: torch.Tensor
    rossby_radii: np.ndarray | None


BaroclinicQGDiagnostics = QGDiagnostics
BarotropicQGDiagnostics = QGDiagnostics


@dataclasses.dataclass(frozen=True)
class BaroclinicQGPhysConsts:
    """Frozen constants of the multilayer model (``baroclinic.py:51-62``)."""

    f0: float = 1e-4
    beta: float = 1.6e-11
    n_layers: int = 2


@dataclasses.dataclass(frozen=True)
class BarotropicQGPhysConsts:
    """Frozen constants of the barotropic model (``barotropic.py:47-58``)."""

    f0: float = 1e-4
    beta: float = 1.6e-11


@dataclasses.dataclass(frozen=True)
class Grid:
    """Arakawa C-grid with one ghost ring (finitevolx ``ArakawaCGrid2D.from_interior``)."""

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


# ---------------------------------------------------------------------------------------
# Plan: one libqgcore plan for one or more members
# ---------------------------------------------------------------------------------------
def _stream_handle(device) -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def lsweep_classes(spec, rows: int) -> set:
    """Strip classes of a member's layer-per-warp sweep items with ``rows``-row strips: 0 =
    every column and row the strip reads strictly inside the member, 1 = edge strip in x and
    y, 2 = masked member, 3 = edge in x only, 4 = edge in y only (one kernel launch per class
    and layer count present)."""
    if spec.mask is not None:
        return {2}
    Ny, Nx = spec.ny + 2, spec.nx + 2
    # row bands: a remainder of fewer than 8 rows joins the last full band (lsweep_bands)
    bands = (Ny + rows - 1) // rows
    rem = Ny - (bands - 1) * rows
    if bands > 1 and rem < 8 and rows + rem <= 64:
        bands -= 1
    out = set()
    for sy in range(bands):
        for sx in range((Nx + 59) // 60):
            x0, jb = 60 * sx, rows * sy
            rhi = (Ny if sy == bands - 1 else jb + rows) + 1
            xin = x0 - 2 >= 1 and x0 + 61 <= Nx - 2
            yin = jb - 2 >= 1 and rhi <= Ny - 2
            out.add((0 if yin else 4) if xin else (3 if yin else 1))
    return out


class Plan:
    """Owns a ``qg_plan`` (device constants + workspace) on one CUDA device."""

    def __init__(self, members: Sequence["MemberSpec"], precision="fp32", refine=0, use_graphs=True,
                 device=None, persistent=True, autotune=True, stencil=None, gemm_tile=None, cluster=None):
        """``cluster``: cluster-resident stepping of small members (``step`` with Heun / SSP-RK3 in
        one launch per call): None = when the autotuner times it faster, True = whenever the
        members allow it, False = never."""
        if not torch.cuda.is_available():
            raise RuntimeError("somax_gb300 needs a CUDA device (no CPU fallback)")
        d = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        if d.type == "cuda" and d.index is None:
            d = torch.device("cuda", torch.cuda.current_device())
        self.device = d
        L = _lib.lib()
        arr = (MemberDesc * len(members))()
        for i, m in enumerate(members):
            m.fill(arr[i])
        forced = 0 if stencil is None else 1 + self.STENCIL_VARIANTS.index(stencil)
        opts = Options(PRECISIONS[precision], int(refine), int(bool(use_graphs)), int(bool(persistent)),
                       int(bool(autotune)), forced, int(gemm_tile or 0), 0 if cluster is None else (1 if cluster else 2))
        handle = C.c_void_p()
        with torch.cuda.device(self.device):
            check(L.qg_plan_create(arr, len(members), C.byref(opts), C.byref(handle)), "qg_plan_create")
        self._h = handle
        self._L = L
        self.members = list(members)
        self.precision = precision
        self.refine = int(refine)
        self.persistent = bool(persistent)
        self.state_size = int(L.qg_plan_state_size(handle))
        self.offsets = [int(L.qg_plan_member_offset(handle, i)) for i in range(len(members))]

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._L.qg_plan_destroy(h)
            except Exception:  # pragma: no cover
                pass
            self._h = None

    @property
    def handle(self):
        return self._h

    def member_modes(self, i: int):
        n = self.members[i].n_layers
        lam = (C.c_double * n)()
        a = (C.c_double * (n * n))()
        b = (C.c_double * (n * n))()
        check(self._L.qg_plan_member_modes(self._h, i, lam, a, b), "qg_plan_member_modes")
        return np.array(lam), np.array(a).reshape(n, n), np.array(b).reshape(n, n)

    def _check_field(self, t: torch.Tensor, name: str):
        if not isinstance(t, torch.Tensor) or t.device.type != "cuda" or t.dtype != torch.float32:
            raise TypeError(f"{name} must be a float32 CUDA tensor")
        if t.device != self.device:
            raise ValueError(f"{name} is on {t.device}, the plan on {self.device}")
        if not t.is_contiguous() or t.numel() != self.state_size:
            raise ValueError(f"{name} must be contiguous with {self.state_size} elements, got {tuple(t.shape)}")

    def invert(self, q: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        self._check_field(q, "q")
        out = torch.empty_like(q) if out is None else out
        self._check_field(out, "psi")
        check(self._L.qg_invert(self._h, C.c_void_p(q.data_ptr()), C.c_void_p(out.data_ptr()),
                                _stream_handle(q.device)), "qg_invert")
        return out

    def rhs(self, q: torch.Tensor, params: torch.Tensor, apply_bc=False, out=None) -> torch.Tensor:
        self._check_field(q, "q")
        out = torch.empty_like(q) if out is None else out
        self._check_field(out, "dq")
        params = params.detach().to(device=q.device, dtype=torch.float32).contiguous()
        if params.numel() != 4 * len(self.members):
            raise ValueError("params must hold 4 values per member")
        flags = K["QG_RHS_APPLY_BC"] if apply_bc else 0
        check(self._L.qg_rhs(self._h, C.c_void_p(q.data_ptr()), C.c_void_p(out.data_ptr()),
                             C.c_void_p(params.data_ptr()), flags, _stream_handle(q.device)), "qg_rhs")
        return out

    def _params(self, params: torch.Tensor, device) -> torch.Tensor:
        params = params.detach().to(device=device, dtype=torch.float32).contiguous()
        if params.numel() != 4 * len(self.members):
            raise ValueError("params must hold 4 values per member")
        return params

    def rhs_vjp(self, q: torch.Tensor, params: torch.Tensor, dq_bar: torch.Tensor, apply_bc=False,
                want_params=True):
        """(q_bar, params_bar) of ``rhs(q, params, apply_bc)`` for the cotangent ``dq_bar``."""
        self._check_field(q, "q")
        self._check_field(dq_bar, "dq_bar")
        params = self._params(params, q.device)
        q_bar = torch.empty_like(q)
        p_bar = torch.empty_like(params) if want_params else None
        flags = K["QG_RHS_APPLY_BC"] if apply_bc else 0
        check(self._L.qg_rhs_vjp(self._h, C.c_void_p(q.data_ptr()), C.c_void_p(params.data_ptr()),
                                 C.c_void_p(dq_bar.data_ptr()), C.c_void_p(q_bar.data_ptr()),
                                 C.c_void_p(p_bar.data_ptr() if p_bar is not None else None), flags,
                                 _stream_handle(q.device)), "qg_rhs_vjp")
        return q_bar, p_bar

    def step_vjp(self, y0: torch.Tensor, params: torch.Tensor, dt: float, scheme: str, g: torch.Tensor,
                 want_params: bool = True):
        """(y0_bar, params_bar) of one ``step`` of ``scheme`` from ``y0`` for the cotangent ``g`` of
        its result (``qg_step_vjp``: stage recomputation and reverse sweep in one call)."""
        self._check_field(y0, "y0")
        self._check_field(g, "g")
        params = self._params(params, y0.device)
        # the call's state, cotangent and parameters go through buffers that stay put from call
        # to call, so that the library replays its captured graph of the step's adjoint
        key = (scheme, y0.device)
        bufs = getattr(self, "_vjp_bufs", {})
        if key not in bufs:
            n = int(self._L.qg_step_vjp_workspace(self._h, SCHEMES[scheme]))
            bufs[key] = dict(work=torch.empty(n, dtype=torch.float32, device=y0.device),
                             y0=torch.empty_like(y0), y_bar=torch.empty_like(y0), params=torch.empty_like(params),
                             p_bar=torch.empty_like(params))
            self._vjp_bufs = bufs
        b = bufs[key]
        b["y0"].copy_(y0)
        b["y_bar"].copy_(g)
        b["params"].copy_(params)
        check(self._L.qg_step_vjp(self._h, C.c_void_p(b["y0"].data_ptr()), C.c_void_p(b["params"].data_ptr()),
                                  float(dt), SCHEMES[scheme], C.c_void_p(b["y_bar"].data_ptr()),
                                  C.c_void_p(b["p_bar"].data_ptr()), C.c_void_p(b["work"].data_ptr()),
                                  _stream_handle(y0.device)), "qg_step_vjp")
        return b["y_bar"].clone(), (b["p_bar"].clone() if want_params else None)

    def invert_vjp(self, psi_bar: torch.Tensor) -> torch.Tensor:
        """q_bar of ``invert(q)`` for the cotangent ``psi_bar`` (the map is linear in q)."""
        self._check_field(psi_bar, "psi_bar")
        q_bar = torch.empty_like(psi_bar)
        check(self._L.qg_invert_vjp(self._h, C.c_void_p(psi_bar.data_ptr()), C.c_void_p(q_bar.data_ptr()),
                                    _stream_handle(psi_bar.device)), "qg_invert_vjp")
        return q_bar

    def step(self, q: torch.Tensor, params: torch.Tensor, dt: float, n_steps: int, scheme: str,
             apply_bc: bool = True) -> torch.Tensor:
        """Advance q in place: BC on every stage input; ``apply_bc`` zeroes the ring of the
        initial state first (a new integrate()), otherwise the call continues one."""
        self._check_field(q, "q")
        params = params.detach().to(device=q.device, dtype=torch.float32).contiguous()
        if params.numel() != 4 * len(self.members):
            raise ValueError("params must hold 4 values per member")
        check(self._L.qg_step(self._h, C.c_void_p(q.data_ptr()), C.c_void_p(params.data_ptr()),
                              float(dt), int(n_steps), SCHEMES[scheme], K["QG_STEP_APPLY_BC"] if apply_bc else 0,
                              _stream_handle(q.device)), "qg_step")
        return q

    def diagnose(self, q: torch.Tensor):
        self._check_field(q, "q")
        nlt = sum(m.n_layers for m in self.members)
        ke = torch.empty(nlt, device=q.device, dtype=torch.float32)
        en = torch.empty(nlt, device=q.device, dtype=torch.float32)
        check(self._L.qg_diagnose(self._h, C.c_void_p(q.data_ptr()), C.c_void_p(ke.data_ptr()),
                                  C.c_void_p(en.data_ptr()), _stream_handle(q.device)), "qg_diagnose")
        return ke, en

    def state_stats(self, q: torch.Tensor) -> torch.Tensor:
        """(min, mean, max) over the finite entries of the packed field q and the count of its
        non-finite entries, as a float64 device tensor of 4 values (``qg_state_stats``)."""
        self._check_field(q, "q")
        out = torch.empty(4, device=q.device, dtype=torch.float64)
        check(self._L.qg_state_stats(self._h, C.c_void_p(q.data_ptr()), C.c_void_p(out.data_ptr()),
                                     _stream_handle(q.device)), "qg_state_stats")
        return out

    def diagnose_fields(self, q: torch.Tensor):
        """(psi, u, v, zeta, ke, ens) of the packed field q from one inversion (``qg_diagnose_fields``)."""
        self._check_field(q, "q")
        psi, u, v, zeta = (torch.empty_like(q) for _ in range(4))
        nlt = sum(m.n_layers for m in self.members)
        ke = torch.empty(nlt, device=q.device, dtype=torch.float32)
        en = torch.empty(nlt, device=q.device, dtype=torch.float32)
        ptr = [C.c_void_p(t.data_ptr()) for t in (q, psi, u, v, zeta, ke, en)]
        check(self._L.qg_diagnose_fields(self._h, *ptr, _stream_handle(q.device)), "qg_diagnose_fields")
        return psi, u, v, zeta, ke, en

    def status(self, device=None) -> int:
        flags = C.c_int(0)
        code = self._L.qg_status(self._h, C.byref(flags), _stream_handle(device or self.device))
        if code not in (0, K["QG_ERR_NONFINITE"], K["QG_ERR_TIMEOUT"]):
            check(code, "qg_status")
        return code

    def launches_per_call(self, n_steps: int, scheme: str) -> int:
        """Kernels libqgcore launches for one ``step`` call of ``n_steps`` steps."""
        stages = {"euler": 1, "heun": 2, "ssprk3": 3, "tsit5": 6}[scheme]
        butcher = scheme in ("euler", "tsit5")
        masked = any(m.mask is not None for m in self.members)
        if self.engine()["cluster_ctas"] and not butcher:
            return 1  # the cluster-resident step kernel, every stage of every step
        if self.persistent and self.precision != "fp32" and self.refine == 0 and not butcher and not masked:
            return 3  # pack, the persistent step kernel, unpack
        # the column-sweep stencils launch once per distinct layer count, the layer-per-warp
        # sweep once per distinct (layer count, strip class)
        variant = self.tuning()["stencil"]
        if variant.startswith("lsweep"):
            rows = int(variant[len("lsweep"):])
            stencil = len({(m.n_layers, c) for m in self.members for c in lsweep_classes(m, rows)})
        elif "sweep" in variant:
            stencil = len({m.n_layers for m in self.members})
        else:
            stencil = 1
        solve = 4 * (1 + self.refine) + self.refine
        inversion = solve
        if masked:  # capacitance correction(s), each followed by a solve
            inversion += (1 + self.refine) * (1 + (1 if self.refine else 0) + solve)
        per_stage = inversion + stencil + (1 if butcher else 0)
        return 2 + n_steps * stages * per_stage

    STENCIL_VARIANTS = ("tile32x8", "tile64x16", "sweep16", "sweep32", "sweep64", "lsweep16", "lsweep32", "lsweep64")

    def tuning(self) -> dict:
        """The autotuner's stencil choice and the time (ms) of one RK stage (four DST passes
        and the stencil) it measured with every variant."""
        v = C.c_int()
        n = len(self.STENCIL_VARIANTS)
        ms = (C.c_float * n)()
        check(self._L.qg_plan_tuning(self._h, C.byref(v), ms, n), "qg_plan_tuning")
        bn = C.c_int()
        gms = (C.c_float * 5)()
        check(self._L.qg_plan_gemm_tuning(self._h, C.byref(bn), gms, 5), "qg_plan_gemm_tuning")
        return {"stencil": self.STENCIL_VARIANTS[v.value],
                "ms": {name: round(float(t), 5) for name, t in zip(self.STENCIL_VARIANTS, ms)},
                "gemm_tile_n": bn.value,
                "gemm_ms": {w: round(float(t), 5) for w, t in zip((144, 80, 48, 32, 16), gms)}}

    def engine(self) -> dict:
        """The stepping engine of ``step`` (Heun / SSP-RK3): the cluster size of the cluster-
        resident engine (0: the multi-launch path) and the autotuner's time (ms) of four SSP-RK3
        steps with each."""
        n = C.c_int()
        ms = (C.c_float * 2)()
        check(self._L.qg_plan_engine(self._h, C.byref(n), ms, 2), "qg_plan_engine")
        return {"cluster_ctas": n.value, "ms": {"multi_launch": round(float(ms[0]), 5),
                                                "cluster": round(float(ms[1]), 5)}}

    def set_wait_limit(self, cycles: int = 0):
        """Clock64 cycles the persistent step kernel waits at a grid barrier before it gives
        up and reports QG_ERR_TIMEOUT through ``status`` (0: the default, about 2 s)."""
        check(self._L.qg_plan_set_wait_limit(self._h, int(cycles)), "qg_plan_set_wait_limit")

    def set_parallel_sweep(self, on: bool = True):
        """Launch the layer-per-warp sweep's (layer count, strip class) groups as parallel
        graph branches (default) or one after another on the call's stream."""
        check(self._L.qg_plan_set_parallel_sweep(self._h, int(bool(on))), "qg_plan_set_parallel_sweep")

    def set_profiling(self, on: bool):
        check(self._L.qg_set_profiling(self._h, int(on)), "qg_set_profiling")

    def kernel_stats(self, kclass: int):
        t = C.c_double()
        n = C.c_int64()
        check(self._L.qg_kernel_stats(self._h, kclass, C.byref(t), C.byref(n)), "qg_kernel_stats")
        return t.value, n.value


@dataclasses.dataclass
class MemberSpec:
    """One member of a plan (fills ``qg_member_desc``)."""

    nx: int
    ny: int
    Lx: float
    Ly: float
    f0: float
    beta: float
    H: Sequence[float]
    g_prime: Sequence[float]
    barotropic: bool = False
    wind_profile: str = "doublegyre"
    eigs: str = "consistent"
    modal: ModalTransform | None = None
    mask: np.ndarray | None = None  # (ny + 2, nx + 2) land mask, 1 = ocean (extension)

    @property
    def n_layers(self) -> int:
        return 1 if self.barotropic else len(self.H)

    @property
    def cells(self) -> int:
        return self.n_layers * (self.nx + 2) * (self.ny + 2)

    def fill(self, d: MemberDesc) -> None:
        n = self.n_layers
        d.nx, d.ny, d.n_layers, d.barotropic = self.nx, self.ny, n, int(self.barotropic)
        d.Lx, d.Ly, d.f0, d.beta = self.Lx, self.Ly, self.f0, self.beta
        for k in range(n):
            d.H[k] = float(self.H[k]) if not self.barotropic else 1.0
            d.g_prime[k] = float(self.g_prime[k]) if not self.barotropic else 1.0
        d.wind_profile = K["QG_WIND_SINGLE"] if self.wind_profile == "single" else K["QG_WIND_DOUBLEGYRE"]
        d.eigs_mode = K["QG_EIGS_REFERENCE"] if self.eigs == "reference" else K["QG_EIGS_CONSISTENT"]
        if self.mask is not None:
            m = np.ascontiguousarray(self.mask, dtype=np.uint8)
            if m.shape != (self.ny + 2, self.nx + 2):
                raise ValueError(f"mask must have shape {(self.ny + 2, self.nx + 2)}, got {m.shape}")
            self._mask_c = m  # kept alive while qg_plan_create reads it
            d.mask = m.ctypes.data_as(C.POINTER(C.c_ubyte))
        if self.modal is not None and not self.barotropic:
            d.has_modes = 1
            lam = self.f0**2 * np.asarray(self.modal.eigenvalues, float)
            for r in range(n):
                d.lambdas[r] = float(lam[r])
                for c in range(n):
                    d.Cl2m[r * n + c] = float(self.modal.Cl2m[r, c])
                    d.Cm2l[r * n + c] = float(self.modal.Cm2l[r, c])


# ---------------------------------------------------------------------------------------
# Models
# ---------------------------------------------------------------------------------------
class SomaxModel:
    """The model contract of ``core/model.py:12-95``."""

    def vector_field(self, t, state, args=None):  # pragma: no cover - abstract
        raise NotImplementedError

    def apply_boundary_conditions(self, state):  # pragma: no cover - abstract
        raise NotImplementedError


def _zero_ring(q: torch.Tensor) -> torch.Tensor:
    out = q.clone()
    out[..., 0, :] = 0
    out[..., -1, :] = 0
    out[..., :, 0] = 0
    out[..., :, -1] = 0
    return out


class _QGBase(SomaxModel):
    state_cls = State
    barotropic = False

    def __init__(self, spec: MemberSpec, params: QGParams, precision="fp32", refine=0, use_graphs=True,
                 strat=None, modal=None, persistent=True, stencil=None, gemm_tile=None, cluster=None):
        self.spec = spec
        self.params = params
        self.precision = precision
        self.refine = refine
        self.use_graphs = use_graphs
        self.persistent = persistent
        self.stencil = stencil
        self.gemm_tile = gemm_tile
        self.cluster = cluster
        self.strat = strat
        self.modal = modal
        self.grid = Grid(spec.nx, spec.ny, spec.Lx, spec.Ly)
        self._plans: dict = {}

    # the plan is created lazily on the device of the first field it sees
    def plan(self, device=None) -> Plan:
        device = torch.device(device if device is not None else "cuda")
        if device.index is None:
            device = torch.device("cuda", torch.cuda.current_device())
        key = device.index
        if key not in self._plans:
            self._plans[key] = Plan([self.spec], self.precision, self.refine, self.use_graphs, device, self.persistent,
                                    stencil=self.stencil, gemm_tile=self.gemm_tile, cluster=self.cluster)
        return self._plans[key]

    @property
    def shape(self):
        g = self.grid
        return (g.Ny, g.Nx) if self.barotropic else (self.spec.n_layers, g.Ny, g.Nx)

    def _field(self, q: torch.Tensor) -> torch.Tensor:
        if tuple(q.shape) != self.shape:
            raise ValueError(f"q must have shape {self.shape}, got {tuple(q.shape)}")
        if q.device.type != "cuda":
            raise TypeError("q must live on a CUDA device")
        return q.to(torch.float32).contiguous()

    def _param_vector(self, device) -> torch.Tensor:
        return self.params.vector(device)

    def _param_tensors(self):
        p = self.params
        return (p.lateral_viscosity, p.bottom_drag, p.wind_amplitude, p.biharmonic_viscosity)

    @staticmethod
    def _grad_needed(*ts) -> bool:
        return torch.is_grad_enabled() and any(isinstance(t, torch.Tensor) and t.requires_grad for t in ts)

    # -- reference API -------------------------------------------------------------------
    def _invert_pv(self, q: torch.Tensor) -> torch.Tensor:
        """psi from q; differentiable in q (hand-written adjoint, ``qg_invert_vjp``)."""
        q = self._field(q)
        plan = self.plan(q.device)
        if self._grad_needed(q):
            return adjoint.invert(plan, q)
        return plan.invert(q)

    def vector_field(self, t, state, args=None):
        """dq/dt for ``state.q`` as given (no BC applied, like the reference); differentiable
        in q and the parameters (hand-written adjoint, ``qg_rhs_vjp``)."""
        q = self._field(state.q)
        pv = self._param_vector(q.device)
        plan = self.plan(q.device)
        if self._grad_needed(q, pv):
            return self.state_cls(q=adjoint.rhs(plan, q, pv, apply_bc=False))
        return self.state_cls(q=plan.rhs(q, pv, apply_bc=False))

    def apply_boundary_conditions(self, state):
        """Zero ring (``baroclinic.py:192-195``); with a land mask, land cells are zeroed too."""
        q = _zero_ring(state.q)
        if self.spec.mask is not None:
            ocean = torch.as_tensor(np.asarray(self.spec.mask) != 0, device=q.device)
            ocean[0, :] = True
            ocean[-1, :] = True
            ocean[:, 0] = True
            ocean[:, -1] = True
            q = q * ocean.to(q.dtype)
        return self.state_cls(q=q)

    def step(self, state, dt: float, n_steps: int = 1, solver="ssprk3", out: torch.Tensor | None = None,
             apply_bc: bool = True):
        """Advance ``n_steps`` constant steps on the GPU; returns a new state.

        Like ``integrate``, the ring of the initial state is zeroed first (``apply_bc``) and
        the BC is applied to every stage input.  A state held in host memory is copied to the
        current CUDA device, stepped there and copied back (into ``out`` if given; pinned
        memory makes both copies asynchronous)."""
        q_in = state.q
        host = q_in.device.type == "cpu"
        if host:
            if tuple(q_in.shape) != self.shape:
                raise ValueError(f"q must have shape {self.shape}, got {tuple(q_in.shape)}")
            dev = torch.device("cuda", torch.cuda.current_device())
            q = q_in.to(device=dev, dtype=torch.float32, non_blocking=True).contiguous()
        else:
            q = self._field(q_in).clone()
        scheme = _solver_name(solver)
        self.plan(q.device).step(q, self._param_vector(q.device), dt, n_steps, scheme, apply_bc)
        if host:
            if out is None:
                out = torch.empty(q.shape, dtype=torch.float32, pin_memory=True)
            out.copy_(q, non_blocking=True)
            return self.state_cls(q=out)
        return self.state_cls(q=q)

    def integrate(self, state0, t0: float, t1: float, dt: float, solver=None, saveat=None, **kw):
        """``SomaxModel.integrate`` with constant steps (``core/model.py:53-88``).

        Differentiable in ``state0.q`` and the parameters: when either requires grad, each
        saved interval runs through the checkpointed adjoint (``checkpoint_every`` steps per
        checkpoint, default 10), as diffrax's recursive-checkpoint adjoint does for the
        reference's ``eqx.filter_grad`` (``tests/models/test_qg_baroclinic.py:293-312``)."""
        if kw.get("stepsize_controller") not in (None, "constant"):
            raise ValueError("only constant step sizes are supported")
        every = int(kw.get("checkpoint_every", 10))
        scheme = _solver_name(solver)
        saveat = saveat or SaveAt(t1=True)
        n_total = int(round((t1 - t0) / dt))
        if abs(n_total * dt - (t1 - t0)) > 1e-9 * max(1.0, abs(t1 - t0)):
            raise ValueError("(t1 - t0) must be a whole number of steps")
        if saveat.ts is not None:
            targets = [int(round((float(t) - t0) / dt)) for t in saveat.ts]
        else:
            targets = [n_total]
        state = self.apply_boundary_conditions(state0)
        ys, done = [], 0
        q = state.q
        pv = None
        grad = self._grad_needed(q) or self._grad_needed(*self._param_tensors())
        if grad:
            q = self._field(q)
            pv = self._param_vector(q.device)
        for tgt in targets:
            if tgt < done:
                raise ValueError("saveat.ts must be increasing")
            if tgt > done:
                # one continuous integration: only the first chunk starts from a BC'd state
                if grad:
                    q = adjoint.integrate(self.plan(q.device), q, pv, dt, tgt - done, scheme, apply_bc=False,
                                          checkpoint_every=every)
                else:
                    q = self.step(self.state_cls(q=q), dt, tgt - done, scheme, apply_bc=False).q
                done = tgt
            ys.append(q.clone())
        ts = torch.tensor([t0 + k * dt for k in targets], dtype=torch.float64)
        return Solution(ts=ts, ys=self.state_cls(q=torch.stack(ys)))

    def diagnose(self, state) -> QGDiagnostics:
        """``diagnose`` (``baroclinic.py:197-228``): psi, u, v, relative vorticity, KE and
        enstrophy per layer, all from one inversion on the GPU (``qg_diagnose_fields``)."""
        q = self._field(state.q)
        plan = self.plan(q.device)
        shp = q.shape
        psi, u, v, zeta, ke, en = plan.diagnose_fields(q.reshape(-1).contiguous())
        radii = None if self.modal is None else self.modal.rossby_radii
        if self.barotropic:
            ke, en = ke[0], en[0]
        return QGDiagnostics(psi=psi.view(shp), u=u.view(shp), v=v.view(shp), kinetic_energy=ke,
                             total_kinetic_energy=ke.sum(), enstrophy=en, total_enstrophy=en.sum(),
                             relative_vorticity=zeta.view(shp), rossby_radii=radii)


class BaroclinicQG(_QGBase):
    """Multilayer QG on an Arakawa C-grid (``baroclinic.py:91-332``)."""

    state_cls = BaroclinicQGState

    @property
    def consts(self) -> BaroclinicQGPhysConsts:
        return BaroclinicQGPhysConsts(f0=self.spec.f0, beta=self.spec.beta, n_layers=self.spec.n_layers)

    @property
    def helmholtz_lambdas(self) -> np.ndarray:
        return self.spec.f0**2 * np.asarray(self.modal.eigenvalues)

    @property
    def beta_y(self) -> np.ndarray:
        g = self.grid
        y = np.arange(g.Ny) * g.dy
        return np.broadcast_to((self.spec.beta * (y - g.Ly / 2.0))[:, None], (g.Ny, g.Nx))

    @staticmethod
    def create(nx=64, ny=64, Lx=4e6, Ly=4e6, f0=9.375e-5, beta=1.754e-11, n_layers=3,
               H=(400.0, 1100.0, 2600.0), g_prime=(9.81, 0.025, 0.0125), stratification=None,
               lateral_viscosity=0.0, bottom_drag=0.0, wind_amplitude=0.0, wind_profile="doublegyre",
               poisson_bc="dst", biharmonic_viscosity=0.0, precision="fp32", refine=0, eigs="consistent",
               use_graphs=True, persistent=True, stencil=None, gemm_tile=None, mask=None,
               cluster=None) -> "BaroclinicQG":
        """``BaroclinicQG.create`` (``baroclinic.py:230-332``) with the same keyword arguments,
        plus ``biharmonic_viscosity`` (extension), ``precision`` of the DST-I GEMMs
        ("fp32", "tf32", "bf16x3"), ``refine`` sweeps, the ``eigs`` mode and whether ``step`` runs
        in one ``persistent`` launch (tensor-core precisions)."""
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
                          eigs, modal, mask)
        params = QGParams(*(torch.tensor(float(v)) for v in (lateral_viscosity, bottom_drag, wind_amplitude,
                                                             biharmonic_viscosity)))
        return BaroclinicQG(spec, params, precision, refine, use_graphs, strat, modal, persistent, stencil, gemm_tile,
                            cluster)

    @property
    def n_layers(self):
        return self.spec.n_layers


class BarotropicQG(_QGBase):
    """Barotropic QG (``barotropic.py:79-248``): Poisson inversion, psi ring kept."""

    state_cls = BarotropicQGState
    barotropic = True

    @property
    def consts(self) -> BarotropicQGPhysConsts:
        return BarotropicQGPhysConsts(f0=self.spec.f0, beta=self.spec.beta)

    @staticmethod
    def create(nx=64, ny=64, Lx=1e6, Ly=1e6, f0=1e-4, beta=1.6e-11, lateral_viscosity=0.0,
               bottom_drag=0.0, wind_amplitude=0.0, wind_profile="doublegyre", biharmonic_viscosity=0.0,
               precision="fp32", refine=0, use_graphs=True, persistent=True, stencil=None,
               gemm_tile=None, mask=None, cluster=None) -> "BarotropicQG":
        """``BarotropicQG.create`` (``barotropic.py:186-248``)."""
        spec = MemberSpec(nx, ny, Lx, Ly, f0, beta, [1.0], [1.0], True, wind_profile, mask=mask)
        params = QGParams(*(torch.tensor(float(v)) for v in (lateral_viscosity, bottom_drag, wind_amplitude,
                                                             biharmonic_viscosity)))
        return BarotropicQG(spec, params, precision, refine, use_graphs, persistent=persistent, stencil=stencil,
                            gemm_tile=gemm_tile, cluster=cluster)


class PlanGroup:
    """Members split into ``groups`` contiguous ranges of about equal cell count, one ``Plan``
    each.  The ranges' packed states are contiguous slices of the whole packed state, so a call
    hands each plan its slice with no copy; ``step`` forks the plans onto their own streams and
    joins them, so that independent members' launches overlap on the GPU (one group's DST passes
    beside another's stencil).  Offers the ``Plan`` methods the ensemble uses."""

    def __init__(self, members: Sequence["MemberSpec"], groups: int, device=None, **plan_kw):
        n = len(members)
        groups = max(1, min(int(groups), n))
        cells = [m.cells for m in members]
        total, bounds, acc = float(sum(cells)), [0], 0.0
        for i, c in enumerate(cells):
            acc += c
            if len(bounds) < groups and i + 1 < n and acc >= total * len(bounds) / groups:
                bounds.append(i + 1)
        bounds.append(n)
        self.ranges = list(zip(bounds[:-1], bounds[1:]))
        self.plans = [Plan(list(members[a:b]), device=device, **plan_kw) for a, b in self.ranges]
        self.device = self.plans[0].device
        self.members = list(members)
        self.state_size = sum(p.state_size for p in self.plans)
        self.bases, base = [], 0
        for p in self.plans:
            self.bases.append(base)
            base += p.state_size
        self.offsets = [b + o for b, p in zip(self.bases, self.plans) for o in p.offsets]
        self.streams = [torch.cuda.Stream(device=self.device) for _ in self.plans]
        self.precision = self.plans[0].precision
        self.refine = self.plans[0].refine
        self.persistent = self.plans[0].persistent

    def _slices(self, q: torch.Tensor, params: torch.Tensor):
        params = params.detach().to(device=q.device, dtype=torch.float32).contiguous()
        for p, b, (lo, hi) in zip(self.plans, self.bases, self.ranges):
            yield p, q[b:b + p.state_size], params[4 * lo:4 * hi]

    def step(self, q, params, dt, n_steps, scheme, apply_bc=True):
        if q.numel() != self.state_size or not q.is_contiguous():
            raise ValueError(f"q must be contiguous with {self.state_size} elements")
        cur = torch.cuda.current_stream(q.device)
        start = torch.cuda.Event()
        start.record(cur)
        for (p, qs, ps), st in zip(list(self._slices(q, params)), self.streams):
            st.wait_event(start)
            with torch.cuda.stream(st):
                p.step(qs, ps, dt, n_steps, scheme, apply_bc)
            done = torch.cuda.Event()
            done.record(st)
            cur.wait_event(done)
        return q

    def rhs(self, q, params, apply_bc=False, out=None):
        out = torch.empty_like(q) if out is None else out
        for (p, qs, ps), b in zip(self._slices(q, params), self.bases):
            p.rhs(qs, ps, apply_bc=apply_bc, out=out[b:b + p.state_size])
        return out

    def invert(self, q, out=None):
        out = torch.empty_like(q) if out is None else out
        for p, b in zip(self.plans, self.bases):
            p.invert(q[b:b + p.state_size], out=out[b:b + p.state_size])
        return out

    def status(self, device=None) -> int:
        codes = [p.status(device) for p in self.plans]
        return next((c for c in codes if c), 0)

    def launches_per_call(self, n_steps: int, scheme: str) -> int:
        return sum(p.launches_per_call(n_steps, scheme) for p in self.plans)

    def tuning(self) -> dict:
        t = dict(self.plans[0].tuning())
        t["groups"] = [{"members": hi - lo, **{k: v for k, v in p.tuning().items() if k in ("stencil", "gemm_tile_n")}}
                       for p, (lo, hi) in zip(self.plans, self.ranges)]
        return t

    def engine(self) -> dict:
        return self.plans[0].engine()

    def set_profiling(self, on: bool):
        for p in self.plans:
            p.set_profiling(on)

    def kernel_stats(self, kclass: int):
        ms = n = 0
        for p in self.plans:
            a, b = p.kernel_stats(kclass)
            ms += a
            n += b
        return ms, n

    def set_parallel_sweep(self, on: bool = True):
        for p in self.plans:
            p.set_parallel_sweep(on)


class QGEnsemble:
    """Many independent members (any mix of grid sizes, layer counts and parameters) advanced
    together: one plan, every launch covers all members (the persistent step kernel for the
    tensor-core precisions); with ``groups`` > 1 the members are split into that many plans
    stepped concurrently on their own streams (``PlanGroup``).  States are packed member after
    member in the reference layout."""

    def __init__(self, models: Sequence[_QGBase], precision="bf16x3", refine=0, use_graphs=True, persistent=True,
                 device=None, stencil=None, gemm_tile=None, cluster=None, groups: int = 1):
        if not models:
            raise ValueError("an ensemble needs at least one member")
        self.models = list(models)
        kw = dict(precision=precision, refine=refine, use_graphs=use_graphs, persistent=persistent, stencil=stencil,
                  gemm_tile=gemm_tile, cluster=cluster)
        if groups > 1:
            self.plan = PlanGroup([m.spec for m in self.models], groups, device=device, **kw)
        else:
            self.plan = Plan([m.spec for m in self.models], device=device, **kw)
        self.offsets = self.plan.offsets
        self.sizes = [int(np.prod(m.shape)) for m in self.models]

    @property
    def state_size(self) -> int:
        return self.plan.state_size

    def params(self, device=None) -> torch.Tensor:
        device = device or self.plan.device
        ts = [t for m in self.models for t in m._param_tensors()]
        if any(isinstance(t, torch.Tensor) and t.requires_grad for t in ts):
            return torch.cat([m._param_vector(device) for m in self.models])
        # every member's parameters in one host-to-device copy
        return torch.tensor([float(t) for t in ts], dtype=torch.float32).to(device)

    def pack(self, qs: Sequence[torch.Tensor]) -> torch.Tensor:
        if len(qs) != len(self.models):
            raise ValueError("one field per member")
        for q, m in zip(qs, self.models):
            if tuple(q.shape) != m.shape:
                raise ValueError(f"member field shape {tuple(q.shape)} != {m.shape}")
        return torch.cat([q.reshape(-1).to(torch.float32) for q in qs]).contiguous()

    def unpack(self, packed: torch.Tensor) -> list:
        return [packed[o:o + n].view(m.shape) for o, n, m in zip(self.offsets, self.sizes, self.models)]

    def rhs(self, packed: torch.Tensor, apply_bc=False) -> torch.Tensor:
        return self.plan.rhs(packed, self.params(packed.device), apply_bc=apply_bc)

    def invert(self, packed: torch.Tensor) -> torch.Tensor:
        return self.plan.invert(packed)

    def step(self, packed: torch.Tensor, dt: float, n_steps: int = 1, solver="ssprk3", apply_bc=True) -> torch.Tensor:
        """Advance every member in place by ``n_steps`` steps of ``dt``."""
        scheme = _solver_name(solver)
        return self.plan.step(packed, self.params(packed.device), dt, n_steps, scheme, apply_bc)

    def step_host(self, packed_host: torch.Tensor, out: torch.Tensor, dt: float, n_steps: int = 1,
                  solver="ssprk3", apply_bc=True) -> torch.Tensor:
        """``step`` for a packed state in (pinned) host memory: copy in, step, copy out."""
        if packed_host.numel() != self.state_size:
            raise ValueError("packed state has the wrong size")
        q = packed_host.reshape(-1).to(device=self.plan.device, dtype=torch.float32, non_blocking=True)
        self.step(q, dt, n_steps, solver, apply_bc)
        out.reshape(-1).copy_(q, non_blocking=True)
        return out
