"""The C ABI library loads and exports every symbol include/qgcore.h declares; argument
validation happens on the host before any CUDA call (no GPU needed)."""

import ctypes as C

import pytest

from somax_gb300 import _lib


@pytest.fixture(scope="module")
def L():
    import __graft_entry__

    __graft_entry__.build()
    return _lib.lib()


def test_exports_every_declared_symbol(L):
    names = _lib.declared_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(L, n), f"libqgcore.so does not export {n}"


def test_strerror(L):
    assert _lib.strerror(0) == "ok"
    assert _lib.strerror(_lib.K["QG_ERR_SHAPE"]) == "bad shape"
    assert _lib.strerror(999) == "unknown error"


def test_struct_layout_matches_header(L):
    # 4 ints, 4 doubles, 2 x 8 doubles, 3 ints (+4 pad), 2 x 64 doubles, 8 doubles, mask pointer
    assert C.sizeof(_lib.MemberDesc) == 16 + 32 + 128 + 16 + 1024 + 64 + 8
    assert _lib.MemberDesc.mask.offset == 16 + 32 + 128 + 16 + 1024 + 64
    assert C.sizeof(_lib.Options) == 32
    # qg_swm_desc: 3 ints (+4 pad), 4 doubles, 2 x 8 doubles, 2 ints
    assert C.sizeof(_lib.SwmDesc) == 16 + 32 + 128 + 8
    assert _lib.SwmDesc.wind_profile.offset == 176


def test_swm_create_validates_before_cuda(L):
    h = C.c_void_p()
    d = _lib.SwmDesc()
    d.nx, d.ny, d.n_layers = 0, 16, 2
    assert L.qg_swm_create(C.byref(d), C.byref(h)) == _lib.K["QG_ERR_SHAPE"]
    d.nx, d.Lx, d.Ly = 16, 1e6, 1e6
    d.H[0] = d.H[1] = 500.0
    d.bc = 7
    assert L.qg_swm_create(C.byref(d), C.byref(h)) == _lib.K["QG_ERR_ARG"]
    assert L.qg_swm_create(None, C.byref(h)) == _lib.K["QG_ERR_NULL"]
    assert L.qg_swm_rhs(None, None, None, None, 0, None) == _lib.K["QG_ERR_NULL"]


def test_plan_create_validates_before_cuda(L):
    h = C.c_void_p()
    d = (_lib.MemberDesc * 1)()
    assert L.qg_plan_create(None, 1, None, C.byref(h)) == _lib.K["QG_ERR_NULL"]
    assert L.qg_plan_create(d, 0, None, C.byref(h)) == _lib.K["QG_ERR_SHAPE"]
    d[0].nx, d[0].ny, d[0].n_layers = 8, 8, 0
    assert L.qg_plan_create(d, 1, None, C.byref(h)) == _lib.K["QG_ERR_SHAPE"]
    d[0].n_layers = 9
    assert L.qg_plan_create(d, 1, None, C.byref(h)) == _lib.K["QG_ERR_SHAPE"]
    d[0].n_layers, d[0].Lx, d[0].Ly = 2, 1e6, 1e6
    d[0].H[0] = d[0].H[1] = 100.0
    d[0].g_prime[0], d[0].g_prime[1] = 9.81, -1.0
    assert L.qg_plan_create(d, 1, None, C.byref(h)) == _lib.K["QG_ERR_ARG"]
    d[0].g_prime[1] = 0.02
    d[0].wind_profile = 7
    assert L.qg_plan_create(d, 1, None, C.byref(h)) == _lib.K["QG_ERR_ARG"]
    d[0].wind_profile = 0
    o = _lib.Options(5, 0, 1, 1, 1)
    assert L.qg_plan_create(d, 1, C.byref(o), C.byref(h)) == _lib.K["QG_ERR_ARG"]
    assert h.value is None


def test_entry_points_reject_null(L):
    assert L.qg_invert(None, None, None, None) == _lib.K["QG_ERR_NULL"]
    assert L.qg_rhs(None, None, None, None, 0, None) == _lib.K["QG_ERR_NULL"]
    assert L.qg_step(None, None, None, 1.0, 1, 2, 0, None) == _lib.K["QG_ERR_NULL"]
    assert L.qg_status(None, None, None) == _lib.K["QG_ERR_NULL"]
    assert L.qg_plan_state_size(None) == -1


def test_every_declared_function_has_a_signature(L):
    """The ctypes binding declares the result and argument types of every entry point of the
    header, so a Python caller never passes a 64-bit pointer through an implicit int."""
    for n in _lib.declared_functions():
        assert getattr(L, n).argtypes is not None, f"{n} has no ctypes signature in somax_gb300/_lib.py"


def test_every_plan_entry_point_rejects_null(L):
    """Every entry point that takes a plan answers a NULL plan (and NULL buffers) with QG_ERR_NULL,
    a size query with -1, before any CUDA call."""
    null = _lib.K["QG_ERR_NULL"]
    n = None
    calls = {
        "qg_rhs_vjp": (n, n, n, n, n, n, 0, n),
        "qg_invert_vjp": (n, n, n, n),
        "qg_step_vjp": (n, n, n, 1.0, _lib.K["QG_SCHEME_SSPRK3"], n, n, n, n),
        "qg_project": (n, n, n, n, n, n, n, n, n),
        "qg_project_vjp": (n, n, n, n, n, n, n, n),
        "qg_diagnose": (n, n, n, n, n),
        "qg_diagnose_fields": (n, n, n, n, n, n, n, n, n),
        "qg_state_stats": (n, n, n, n),
        "qg_set_profiling": (n, 1),
        "qg_kernel_stats": (n, 0, n, n),
        "qg_plan_tuning": (n, n, n, 0),
        "qg_plan_gemm_tuning": (n, n, n, 0),
        "qg_plan_engine": (n, n, n, 0),
        "qg_plan_member_modes": (n, 0, n, n, n),
        "qg_plan_set_wait_limit": (n, 100),
        "qg_plan_set_parallel_sweep": (n, 1),
        "qg_invert_static": (n, n, n, n),
        "qg_swm_rhs": (n, n, n, n, 0, n),
        "qg_swm_apply_bc": (n, n, n),
        "qg_swm_step": (n, n, n, 1.0, 1, _lib.K["QG_SCHEME_TSIT5"], 0, n),
        "qg_swm_rhs_vjp": (n, n, n, n, n, n, 0, n),
        "qg_swm_bc_vjp": (n, n, n),
        "qg_swm_step_vjp": (n, n, n, 1.0, _lib.K["QG_SCHEME_TSIT5"], n, n, n, n),
        "qg_swm_segment_vjp": (n, n, n, 1.0, 2, _lib.K["QG_SCHEME_TSIT5"], n, n, n, n),
        "qg_swm_state_stats": (n, n, 4, n, n),
        "qg_swm_set_profiling": (n, 1),
        "qg_swm_kernel_stats": (n, 0, n, n),
        "qg_swm_set_engine": (n, 0),
        "qg_swm_status": (n, n, n),
        "qg_reparam_step": (n, n, n, n, 1.0, 1, _lib.K["QG_SCHEME_TSIT5"], 0, n),
        "qg_reparam_bc_vjp": (n, n, n, n),
        "qg_reparam_step_vjp": (n, n, n, n, 1.0, _lib.K["QG_SCHEME_TSIT5"], n, n, n, n),
    }
    for name, args in calls.items():
        assert getattr(L, name)(*args) == null, name
    assert L.qg_swm_engine(None, _lib.K["QG_SCHEME_TSIT5"], None, None) == -null
    sizes = {
        "qg_plan_member_offset": (n, 0),
        "qg_step_vjp_workspace": (n, _lib.K["QG_SCHEME_SSPRK3"]),
        "qg_swm_state_size": (n,),
        "qg_swm_step_vjp_workspace": (n, _lib.K["QG_SCHEME_TSIT5"]),
        "qg_swm_segment_vjp_workspace": (n, _lib.K["QG_SCHEME_TSIT5"], 2),
        "qg_reparam_step_vjp_workspace": (n, _lib.K["QG_SCHEME_TSIT5"]),
    }
    for name, args in sizes.items():
        assert getattr(L, name)(*args) == -1, name
    L.qg_plan_destroy(None)
    L.qg_swm_destroy(None)
