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
