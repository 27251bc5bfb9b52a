"""ctypes binding of libqgcore.so (the C ABI declared in include/qgcore.h).

The library is the only compute path: if it is missing or fails to load, every call raises
``QGLibraryError``; there is no CPU fallback.
"""

from __future__ import annotations

import ctypes as C
import pathlib
import re

LIB_PATH = pathlib.Path(__file__).resolve().parent / "lib" / "libqgcore.so"
HEADER = pathlib.Path(__file__).resolve().parent.parent / "include" / "qgcore.h"


class QGLibraryError(RuntimeError):
    pass


class QGError(RuntimeError):
    """A QG_ERR_* status returned by the library."""

    def __init__(self, code: int, what: str):
        self.code = code
        super().__init__(f"{what}: {strerror(code)} (code {code})")


def _constants() -> dict:
    out = {}
    for name, val in re.findall(r"#define\s+(QG_[A-Z0-9_]+)\s+(-?\d+)", HEADER.read_text()):
        out[name] = int(val)
    return out


K = _constants()
MAX_LAYERS = K["QG_MAX_LAYERS"]


class MemberDesc(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("n_layers", C.c_int), ("barotropic", C.c_int),
        ("Lx", C.c_double), ("Ly", C.c_double), ("f0", C.c_double), ("beta", C.c_double),
        ("H", C.c_double * MAX_LAYERS), ("g_prime", C.c_double * MAX_LAYERS),
        ("wind_profile", C.c_int), ("eigs_mode", C.c_int), ("has_modes", C.c_int),
        ("Cl2m", C.c_double * (MAX_LAYERS * MAX_LAYERS)),
        ("Cm2l", C.c_double * (MAX_LAYERS * MAX_LAYERS)),
        ("lambdas", C.c_double * MAX_LAYERS),
        ("mask", C.POINTER(C.c_ubyte)),
    ]


class SwmDesc(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("n_layers", C.c_int),
        ("Lx", C.c_double), ("Ly", C.c_double), ("f0", C.c_double), ("beta", C.c_double),
        ("H", C.c_double * MAX_LAYERS), ("g_prime", C.c_double * MAX_LAYERS),
        ("wind_profile", C.c_int), ("bc", C.c_int),
    ]


class Options(C.Structure):
    _fields_ = [("dst_precision", C.c_int), ("refine_sweeps", C.c_int), ("use_graphs", C.c_int),
                ("persistent", C.c_int), ("autotune", C.c_int), ("stencil", C.c_int),
                ("gemm_tile", C.c_int), ("cluster", C.c_int)]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise QGLibraryError(f"{LIB_PATH} is not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
    try:
        L = C.CDLL(str(LIB_PATH))
    except OSError as e:  # pragma: no cover
        raise QGLibraryError(f"cannot load {LIB_PATH}: {e}") from e
    vp, i64 = C.c_void_p, C.c_int64
    sig = {
        "qg_plan_create": (C.c_int, [C.POINTER(MemberDesc), C.c_int, C.POINTER(Options), C.POINTER(vp)]),
        "qg_plan_destroy": (None, [vp]),
        "qg_plan_state_size": (i64, [vp]),
        "qg_plan_member_offset": (i64, [vp, C.c_int]),
        "qg_plan_member_modes": (C.c_int, [vp, C.c_int, vp, vp, vp]),
        "qg_invert": (C.c_int, [vp, vp, vp, vp]),
        "qg_invert_static": (C.c_int, [C.POINTER(MemberDesc), vp, vp, vp]),
        "qg_rhs": (C.c_int, [vp, vp, vp, vp, C.c_int, vp]),
        "qg_step": (C.c_int, [vp, vp, vp, C.c_double, C.c_int, C.c_int, C.c_int, vp]),
        "qg_rhs_vjp": (C.c_int, [vp, vp, vp, vp, vp, vp, C.c_int, vp]),
        "qg_invert_vjp": (C.c_int, [vp, vp, vp, vp]),
        "qg_diagnose": (C.c_int, [vp, vp, vp, vp, vp]),
        "qg_status": (C.c_int, [vp, C.POINTER(C.c_int), vp]),
        "qg_strerror": (C.c_char_p, [C.c_int]),
        "qg_set_profiling": (C.c_int, [vp, C.c_int]),
        "qg_kernel_stats": (C.c_int, [vp, C.c_int, C.POINTER(C.c_double), C.POINTER(i64)]),
        "qg_plan_tuning": (C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_float), C.c_int]),
        "qg_plan_gemm_tuning": (C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_float), C.c_int]),
        "qg_plan_engine": (C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_float), C.c_int]),
        "qg_project": (C.c_int, [vp, vp, vp, vp, vp, vp, vp, vp, vp]),
        "qg_plan_set_wait_limit": (C.c_int, [vp, i64]),
        "qg_state_stats": (C.c_int, [vp, vp, vp, vp]),
        "qg_diagnose_fields": (C.c_int, [vp, vp, vp, vp, vp, vp, vp, vp, vp]),
        "qg_step_vjp_workspace": (i64, [vp, C.c_int]),
        "qg_step_vjp": (C.c_int, [vp, vp, vp, C.c_double, C.c_int, vp, vp, vp, vp]),
        "qg_swm_create": (C.c_int, [C.POINTER(SwmDesc), C.POINTER(vp)]),
        "qg_swm_destroy": (None, [vp]),
        "qg_swm_state_size": (i64, [vp]),
        "qg_swm_rhs": (C.c_int, [vp, vp, vp, vp, C.c_int, vp]),
        "qg_swm_apply_bc": (C.c_int, [vp, vp, vp]),
        "qg_swm_step": (C.c_int, [vp, vp, vp, C.c_double, C.c_int, C.c_int, C.c_int, vp]),
        "qg_reparam_step": (C.c_int, [vp, vp, vp, vp, C.c_double, C.c_int, C.c_int, C.c_int, vp]),
        "qg_swm_set_profiling": (C.c_int, [vp, C.c_int]),
        "qg_swm_set_engine": (C.c_int, [vp, C.c_int]),
        "qg_swm_state_stats": (C.c_int, [vp, vp, C.c_int64, vp, vp]),
        "qg_swm_rhs_vjp": (C.c_int, [vp, vp, vp, vp, vp, vp, C.c_int, vp]),
        "qg_swm_bc_vjp": (C.c_int, [vp, vp, vp]),
        "qg_swm_step_vjp_workspace": (C.c_int64, [vp, C.c_int]),
        "qg_swm_step_vjp": (C.c_int, [vp, vp, vp, C.c_double, C.c_int, vp, vp, vp, vp]),
        "qg_swm_segment_vjp_workspace": (C.c_int64, [vp, C.c_int, C.c_int]),
        "qg_swm_segment_vjp": (C.c_int, [vp, vp, vp, C.c_double, C.c_int, C.c_int, vp, vp, vp, vp]),
        "qg_project_vjp": (C.c_int, [vp, vp, vp, vp, vp, vp, vp, vp]),
        "qg_reparam_bc_vjp": (C.c_int, [vp, vp, vp, vp]),
        "qg_reparam_step_vjp_workspace": (C.c_int64, [vp, C.c_int]),
        "qg_reparam_step_vjp": (C.c_int, [vp, vp, vp, vp, C.c_double, C.c_int, vp, vp, vp, vp]),
        "qg_swm_engine": (C.c_int, [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_float)]),
        "qg_swm_kernel_stats": (C.c_int, [vp, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
        "qg_swm_status": (C.c_int, [vp, C.POINTER(C.c_int), vp]),
        "qg_plan_set_parallel_sweep": (C.c_int, [vp, C.c_int]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def strerror(code: int) -> str:
    return lib().qg_strerror(code).decode()


def check(code: int, what: str) -> None:
    if code != 0:
        raise QGError(code, what)


def declared_functions() -> list[str]:
    """Function names declared in include/qgcore.h (for the ABI export test)."""
    txt = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(qg_[a-z0-9_]+)\s*\(", txt)))
