"""Restart / snapshot stores (``somax_gb300.io``), restating the reference's
``tests/test_io_xarray.py`` for the states of this package, plus the on-disk zarr layout.

CPU only: the stores are written and read with numpy."""

import gzip
import json

import numpy as np
import pytest
import torch

import somax_gb300 as sg
from somax_gb300 import io


def bc_state(nl=3, ny=6, nx=8, fill=None):
    q = torch.arange(nl * ny * nx, dtype=torch.float32).reshape(nl, ny, nx) if fill is None else \
        torch.full((nl, ny, nx), float(fill))
    return sg.BaroclinicQGState(q=q)


# ---- single states (test_io_xarray.py TestSingleState) ---------------------------------
def test_bc_qg_3d_round_trip_in_memory():
    s = bc_state()
    ds = io.state_to_dataset(s)
    assert ds["q"].dims == ("layer", "y", "x")
    assert ds["q"].shape == (3, 6, 8)
    assert ds.attrs["state_class"] == "BaroclinicQGState"
    r = io.dataset_to_state(ds, sg.BaroclinicQGState)
    assert torch.equal(r.q, s.q)


def test_bt_qg_2d_round_trip():
    s = sg.BarotropicQGState(q=torch.randn(8, 12))
    ds = io.state_to_dataset(s)
    assert ds["q"].dims == ("y", "x")
    assert torch.equal(io.dataset_to_state(ds, sg.BarotropicQGState).q, s.q)


def test_swm_state_round_trip():
    s = sg.MultilayerSW2DState(h=torch.ones(2, 6, 8) * 100.0, u=torch.zeros(2, 6, 8), v=torch.randn(2, 6, 8))
    ds = io.state_to_dataset(s)
    assert set(ds.data_vars) == {"h", "u", "v"}
    r = io.dataset_to_state(ds)
    assert isinstance(r, sg.MultilayerSW2DState)
    for k in "huv":
        assert torch.equal(getattr(r, k), getattr(s, k))


def test_with_explicit_time_adds_singleton_axis():
    ds = io.state_to_dataset(bc_state(), time=42.0)
    assert ds["q"].dims == ("time", "layer", "y", "x")
    assert ds["q"].shape == (1, 3, 6, 8)
    assert "time" in ds.coords
    np.testing.assert_array_equal(ds["time"].values, np.array([42.0]))


def test_extra_attrs_are_merged():
    ds = io.state_to_dataset(bc_state(), attrs={"experiment": "smoke", "config_hash": "abc"})
    assert ds.attrs["experiment"] == "smoke" and ds.attrs["config_hash"] == "abc"
    assert ds.attrs["state_class"] == "BaroclinicQGState"


def test_dataset_to_state_auto_recovers_class():
    s = bc_state()
    r = io.dataset_to_state(io.state_to_dataset(s))
    assert isinstance(r, sg.BaroclinicQGState)
    assert torch.equal(r.q, s.q)


def test_dataset_to_state_missing_attrs_raises():
    ds = io.Dataset({"q": (("y", "x"), np.zeros((4, 4)))})
    with pytest.raises(ValueError, match="state_class"):
        io.dataset_to_state(ds)


def test_dataset_to_state_missing_variable_raises():
    ds = io.Dataset({"h": (("y", "x"), np.zeros((4, 4)))})
    with pytest.raises(ValueError, match="missing variable 'u'"):
        io.dataset_to_state(ds, sg.MultilayerSW2DState)


# ---- snapshots (TestSnapshots) ----------------------------------------------------------
def test_stacked_snapshots_and_time_index():
    nt = 5
    snaps = sg.BaroclinicQGState(q=torch.arange(nt * 2 * 4 * 6, dtype=torch.float32).reshape(nt, 2, 4, 6))
    ts = np.linspace(0.0, 4.0, nt)
    ds = io.snapshots_to_dataset(snaps, ts)
    assert ds["q"].dims == ("time", "layer", "y", "x")
    np.testing.assert_array_equal(ds["time"].values, ts)
    last = io.dataset_to_state(ds)
    assert torch.equal(last.q, snaps.q[-1])
    second = io.dataset_to_state(ds, time_index=1)
    assert torch.equal(second.q, snaps.q[1])


def test_snapshots_leading_dim_mismatch_raises():
    snaps = sg.BaroclinicQGState(q=torch.zeros(3, 2, 4, 4))
    with pytest.raises(ValueError, match="leading dim"):
        io.snapshots_to_dataset(snaps, np.arange(4.0))
    with pytest.raises(ValueError, match="1-D"):
        io.snapshots_to_dataset(snaps, np.zeros((3, 1)))


# ---- zarr stores (TestZarrRoundTrip) ----------------------------------------------------
@pytest.mark.parametrize("fmt", [3, 2])
def test_state_save_load_round_trip(tmp_path, fmt):
    s = bc_state()
    store = tmp_path / "final_state.zarr"
    io.save_dataset(io.state_to_dataset(s, attrs={"experiment": "test"}), store, zarr_format=fmt)
    assert store.is_dir()
    loaded = io.load_dataset(store)
    r = io.dataset_to_state(loaded)
    assert isinstance(r, sg.BaroclinicQGState)
    assert torch.equal(r.q, s.q)
    assert loaded.attrs["experiment"] == "test"
    assert loaded["q"].dims == ("layer", "y", "x")


@pytest.mark.parametrize("fmt", [3, 2])
def test_snapshots_save_load_round_trip_and_append(tmp_path, fmt):
    nt, nl, ny, nx = 3, 2, 6, 8
    snaps = sg.BaroclinicQGState(q=torch.arange(nt * nl * ny * nx, dtype=torch.float32).reshape(nt, nl, ny, nx))
    ts = np.linspace(0.0, 2.0, nt)
    store = tmp_path / "snapshots.zarr"
    io.save_dataset(io.snapshots_to_dataset(snaps, ts), store, zarr_format=fmt)
    loaded = io.load_dataset(store)
    np.testing.assert_array_equal(loaded["q"].values, snaps.q.numpy())
    np.testing.assert_array_equal(loaded["time"].values, ts)
    more = sg.BaroclinicQGState(q=torch.full((2, nl, ny, nx), 7.0))
    io.append_to_dataset(io.snapshots_to_dataset(more, np.array([3.0, 4.0])), store, append_dim="time")
    loaded = io.load_dataset(store)
    assert loaded["q"].shape == (nt + 2, nl, ny, nx)
    np.testing.assert_array_equal(loaded["time"].values, [0.0, 1.0, 2.0, 3.0, 4.0])
    np.testing.assert_array_equal(loaded["q"].values[:nt], snaps.q.numpy())
    assert np.all(loaded["q"].values[nt:] == 7.0)


def test_save_modes(tmp_path):
    store = tmp_path / "s.zarr"
    io.save_dataset(io.state_to_dataset(bc_state(fill=1)), store)
    with pytest.raises(FileExistsError):
        io.save_dataset(io.state_to_dataset(bc_state(fill=2)), store, mode="w-")
    io.save_dataset(io.state_to_dataset(bc_state(fill=3)), store, mode="w")
    assert np.all(io.load_dataset(store)["q"].values == 3.0)


def test_v3_layout_on_disk(tmp_path):
    """The store is a zarr v3 group: root zarr.json with the attrs, one array per variable
    with dimension_names, chunk keys c/i/j/k, little-endian bytes codec."""
    store = tmp_path / "snap.zarr"
    snaps = sg.BaroclinicQGState(q=torch.arange(2 * 3 * 4 * 5, dtype=torch.float32).reshape(2, 3, 4, 5))
    io.save_dataset(io.snapshots_to_dataset(snaps, np.array([0.0, 1.0])), store)
    g = json.loads((store / "zarr.json").read_text())
    assert g["zarr_format"] == 3 and g["node_type"] == "group"
    assert g["attributes"]["state_class"] == "BaroclinicQGState"
    assert g["attributes"]["state_module"] == "somax_gb300.qg"
    a = json.loads((store / "q" / "zarr.json").read_text())
    assert a["node_type"] == "array" and a["shape"] == [2, 3, 4, 5] and a["data_type"] == "float32"
    assert a["dimension_names"] == ["time", "layer", "y", "x"]
    assert a["chunk_grid"]["configuration"]["chunk_shape"] == [1, 3, 4, 5]
    assert a["codecs"] == [{"name": "bytes", "configuration": {"endian": "little"}}]
    raw = (store / "q" / "c" / "1" / "0" / "0" / "0").read_bytes()
    np.testing.assert_array_equal(np.frombuffer(raw, "<f4").reshape(3, 4, 5), snaps.q[1].numpy())


def test_reads_gzip_multichunk_v3_store(tmp_path):
    """A v3 store laid out as zarr-python writes one with the gzip codec and a chunk grid that
    does not divide the shape (edge chunks padded, one chunk missing = fill value)."""
    store = tmp_path / "ext.zarr"
    (store / "q").mkdir(parents=True)
    (store / "zarr.json").write_text(json.dumps({"zarr_format": 3, "node_type": "group", "attributes": {
        "state_class": "BaroclinicQGState", "state_module": "somax._src.models.qg.baroclinic"}}))
    full = np.arange(2 * 5 * 7, dtype=np.float32).reshape(2, 5, 7)
    (store / "q" / "zarr.json").write_text(json.dumps({
        "zarr_format": 3, "node_type": "array", "shape": [2, 5, 7], "data_type": "float32",
        "chunk_grid": {"name": "regular", "configuration": {"chunk_shape": [2, 3, 4]}},
        "chunk_key_encoding": {"name": "default", "configuration": {"separator": "/"}},
        "fill_value": -1.0, "codecs": [{"name": "bytes", "configuration": {"endian": "little"}},
                                       {"name": "gzip", "configuration": {"level": 5}}],
        "attributes": {}, "dimension_names": ["layer", "y", "x"]}))
    expect = np.full_like(full, -1.0)
    for j in range(2):
        for i in range(2):
            if (j, i) == (1, 1):
                continue  # missing chunk
            blk = np.zeros((2, 3, 4), np.float32)
            part = full[:, 3 * j:3 * j + 3, 4 * i:4 * i + 4]
            blk[:, :part.shape[1], :part.shape[2]] = part
            expect[:, 3 * j:3 * j + 3, 4 * i:4 * i + 4] = part
            p = store / "q" / "c" / "0" / str(j) / str(i)
            p.parent.mkdir(parents=True, exist_ok=True)
            p.write_bytes(gzip.compress(blk.tobytes()))
    ds = io.load_dataset(store)
    np.testing.assert_array_equal(ds["q"].values, expect)
    # a store the reference wrote restores into this package's class of the same name
    r = io.dataset_to_state(ds)
    assert isinstance(r, sg.BaroclinicQGState)


# ---- allowlisted auto-import (TestAutoImportAllowlist) ----------------------------------
def _tampered(tmp_path, module):
    store = tmp_path / "tampered.zarr"
    io.save_dataset(io.Dataset({"h": (("y", "x"), np.zeros((4, 4)))},
                               attrs={"state_class": "Whatever", "state_module": module}), store)
    return io.load_dataset(store)


@pytest.mark.parametrize("module", ["os", "somaxxx.evil", "somax_gb300x.evil"])
def test_non_package_module_rejected(tmp_path, module):
    with pytest.raises(ValueError, match="refusing to auto-import"):
        io.dataset_to_state(_tampered(tmp_path, module))


def test_explicit_state_class_bypasses_allowlist(tmp_path):
    with pytest.raises(ValueError, match="missing variable"):
        io.dataset_to_state(_tampered(tmp_path, "os"), state_class=sg.MultilayerSW2DState)


def test_save_state_load_state(tmp_path):
    s = bc_state()
    io.save_state(s, tmp_path / "final_state.zarr", time=86400.0)
    r = io.load_state(tmp_path / "final_state.zarr")
    assert torch.equal(r.q, s.q)
