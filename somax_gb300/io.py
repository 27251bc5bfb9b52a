"""Restart and snapshot files of model states: the zarr stores of ``somax.io``.

Mirrors ``somax/_src/io/xarray.py`` (``state_to_dataset`` :73-117, ``snapshots_to_dataset``
:120-176, ``dataset_to_state`` :179-241, ``save_dataset`` :244-257, ``load_dataset`` :260-272,
``append_to_dataset`` :275-292) without xarray or zarr, which are installed neither here nor on
the GPU hosts: a ``Dataset`` holds named variables with dimension names, coordinates and attrs,
and the store is written and read with numpy and the standard library.

On-disk format (zarr v3, as ``save_dataset`` writes with ``zarr_format=3``): the store is a
directory with a group ``zarr.json`` (``attributes`` = the dataset attrs, among them
``state_class`` / ``state_module``), and one sub-directory per variable with an array
``zarr.json`` (``shape``, ``data_type``, a regular chunk grid, the default chunk-key encoding
``c/i/j/k``, ``dimension_names``) and its chunk files.  Variables with a ``time`` axis are
chunked one time slice per chunk, so ``append_to_dataset`` adds chunk files and rewrites the
shape.  Chunks are written with the ``bytes`` codec (little endian, uncompressed); the reader
also takes ``gzip`` chunks, and ``zstd`` ones when the ``zstandard`` package is importable.
zarr v2 stores (``.zgroup`` / ``.zattrs`` / ``.zarray`` with ``_ARRAY_DIMENSIONS``) are read
as well, and written with ``save_dataset(..., zarr_format=2)``.

Canonical dimension names follow the reference: rank 1 ``(x,)``, rank 2 ``(y, x)``, rank 3
``(layer, y, x)``, with ``time`` prepended for snapshots.  ``dataset_to_state`` recovers the
state class from the attrs only for modules of this package or of ``somax`` (a file the
reference wrote maps to the class of the same name here); anything else needs an explicit
``state_class``, as in the reference (loading a store must not import arbitrary modules).
"""

from __future__ import annotations

import dataclasses
import gzip
import importlib
import json
import math
import shutil
import zlib
from pathlib import Path
from typing import Any

import numpy as np

_DIM_NAMES_BY_RANK = {1: ("x",), 2: ("y", "x"), 3: ("layer", "y", "x")}
_ALLOWED_ROOTS = ("somax_gb300", "somax")


def _infer_dims(rank: int, *, time_axis: bool) -> tuple:
    base = _DIM_NAMES_BY_RANK.get(rank) or tuple(f"dim{i}" for i in range(rank))
    return ("time", *base) if time_axis else base


def _to_numpy(x) -> np.ndarray:
    if hasattr(x, "detach"):  # torch tensors, on any device
        x = x.detach().cpu().numpy()
    return np.asarray(x)


@dataclasses.dataclass
class Variable:
    """One named array with its dimension names (an ``xarray.DataArray`` stand-in)."""

    dims: tuple
    values: np.ndarray
    attrs: dict = dataclasses.field(default_factory=dict)

    def __post_init__(self):
        self.dims = tuple(self.dims)
        self.values = np.asarray(self.values)
        if self.values.ndim != len(self.dims):
            raise ValueError(f"{len(self.dims)} dimension names for an array of rank {self.values.ndim}")

    @property
    def shape(self) -> tuple:
        return self.values.shape

    @property
    def dtype(self):
        return self.values.dtype

    def isel(self, **index) -> "Variable":
        vals, dims = self.values, list(self.dims)
        for name, i in index.items():
            ax = dims.index(name)
            vals = np.take(vals, i, axis=ax)
            if np.ndim(i) == 0:
                dims.pop(ax)
        return Variable(tuple(dims), vals, dict(self.attrs))


class Dataset:
    """Data variables and coordinates (both ``Variable``) plus attrs: the part of
    ``xarray.Dataset`` that the state round trips use."""

    def __init__(self, data_vars: dict | None = None, coords: dict | None = None, attrs: dict | None = None):
        self.data_vars = {k: v if isinstance(v, Variable) else Variable(*v) for k, v in (data_vars or {}).items()}
        self.coords = {k: v if isinstance(v, Variable) else Variable(*v) for k, v in (coords or {}).items()}
        self.attrs = dict(attrs or {})
        sizes = {}
        for name, v in self.variables.items():
            for d, n in zip(v.dims, v.shape):
                if sizes.setdefault(d, n) != n:
                    raise ValueError(f"dimension {d!r} has size {sizes[d]} and {n} (variable {name!r})")
        self.sizes = sizes

    @property
    def variables(self) -> dict:
        return {**self.coords, **self.data_vars}

    @property
    def dims(self) -> dict:
        return dict(self.sizes)

    def __getitem__(self, name: str) -> Variable:
        return self.variables[name]

    def __contains__(self, name: str) -> bool:
        return name in self.variables

    def isel(self, **index) -> "Dataset":
        def sel(vs):
            return {k: (v.isel(**{d: i for d, i in index.items() if d in v.dims})) for k, v in vs.items()}

        return Dataset(sel(self.data_vars), sel(self.coords), self.attrs)


# ---------------------------------------------------------------------------------------
# States <-> datasets
# ---------------------------------------------------------------------------------------
def _state_fields(cls) -> list:
    return [f.name for f in dataclasses.fields(cls)]


def _state_attrs(cls) -> dict:
    return {"state_class": cls.__name__, "state_module": cls.__module__}


def state_to_dataset(state, *, time: float | None = None, attrs: dict | None = None) -> Dataset:
    """One state as a dataset: every field a variable with the canonical dimension names; with
    ``time`` a singleton ``time`` axis and coordinate are prepended (``xarray.py:73-117``)."""
    data_vars = {}
    for name in _state_fields(type(state)):
        leaf = _to_numpy(getattr(state, name))
        dims = _infer_dims(leaf.ndim, time_axis=time is not None)
        data_vars[name] = Variable(dims, leaf[None] if time is not None else leaf)
    coords = {"time": Variable(("time",), np.asarray([time], np.float64))} if time is not None else {}
    return Dataset(data_vars, coords, {**_state_attrs(type(state)), **(attrs or {})})


def snapshots_to_dataset(snapshots, ts, *, state_class=None, attrs: dict | None = None) -> Dataset:
    """Time-stacked states (every field with a leading time axis, as ``integrate(...).ys``) as a
    dataset with a ``time`` coordinate (``xarray.py:120-176``)."""
    state_class = state_class or type(snapshots)
    ts = _to_numpy(ts)
    if ts.ndim != 1:
        raise ValueError(f"ts must be 1-D, got shape {ts.shape}")
    data_vars = {}
    for name in _state_fields(state_class):
        leaf = _to_numpy(getattr(snapshots, name))
        if leaf.shape[0] != ts.shape[0]:
            raise ValueError(f"snapshot leaf {name!r} has leading dim {leaf.shape[0]} but ts has length {ts.shape[0]}")
        data_vars[name] = Variable(_infer_dims(leaf.ndim - 1, time_axis=True), leaf)
    return Dataset(data_vars, {"time": Variable(("time",), ts)}, {**_state_attrs(state_class), **(attrs or {})})


def _resolve_state_class(ds: Dataset):
    try:
        module_name, class_name = ds.attrs["state_module"], ds.attrs["state_class"]
    except KeyError as exc:
        raise ValueError("dataset_to_state called without state_class and the Dataset is missing "
                         "'state_class'/'state_module' attrs") from exc
    root = module_name.split(".")[0]
    if root not in _ALLOWED_ROOTS or (module_name != root and not module_name.startswith(root + ".")):
        raise ValueError(f"refusing to auto-import state_module {module_name!r}: only modules under "
                         f"{' or '.join(repr(r + '.') for r in _ALLOWED_ROOTS)} are allowlisted for "
                         f"auto-recovery. Pass state_class explicitly to load this dataset.")
    if root == "somax":
        # a store the reference wrote: the class of the same name in this package
        pkg = importlib.import_module("somax_gb300")
        if not hasattr(pkg, class_name):
            raise ValueError(f"no state class {class_name!r} in somax_gb300 for the reference's {module_name!r}")
        return getattr(pkg, class_name)
    return getattr(importlib.import_module(module_name), class_name)


def dataset_to_state(ds: Dataset, state_class=None, *, time_index: int = -1, device=None):
    """The state a dataset holds (``xarray.py:179-241``); with a ``time`` axis the slice
    ``time_index`` (default: the last, for a restart).  Fields become float32 torch tensors,
    on ``device`` if given."""
    import torch

    state_class = state_class or _resolve_state_class(ds)
    kwargs = {}
    for name in _state_fields(state_class):
        if name not in ds.variables:
            raise ValueError(f"Dataset is missing variable {name!r} required by {state_class.__name__}")
        var = ds[name]
        if "time" in var.dims:
            var = var.isel(time=time_index)
        t = torch.from_numpy(np.ascontiguousarray(var.values))
        kwargs[name] = t.to(device) if device is not None else t
    return state_class(**kwargs)


# ---------------------------------------------------------------------------------------
# zarr stores
# ---------------------------------------------------------------------------------------
_V3_TYPES = {"bool": "bool", "int8": "int8", "int16": "int16", "int32": "int32", "int64": "int64",
             "uint8": "uint8", "uint16": "uint16", "uint32": "uint32", "uint64": "uint64",
             "float16": "float16", "float32": "float32", "float64": "float64"}


def _json_fill(x):
    if isinstance(x, float) and math.isnan(x):
        return "NaN"
    if isinstance(x, float) and math.isinf(x):
        return "Infinity" if x > 0 else "-Infinity"
    return x


def _parse_fill(x, dtype):
    if isinstance(x, str):
        x = {"NaN": float("nan"), "Infinity": float("inf"), "-Infinity": float("-inf")}.get(x, x)
    return np.asarray(0 if x is None else x).astype(dtype)


def _chunk_shape(var: Variable) -> tuple:
    return tuple(1 if d == "time" else n for d, n in zip(var.dims, var.shape))


def _chunk_indices(shape, chunks):
    grid = [max(1, -(-n // c)) for n, c in zip(shape, chunks)]
    return list(np.ndindex(*grid)) if grid else [()]


def _write_json(path: Path, obj) -> None:
    path.write_text(json.dumps(obj, indent=2, allow_nan=False))


def _write_array(root: Path, name: str, var: Variable, fmt: int, start_chunk: int = 0) -> None:
    """Write the chunks of ``var`` (and its metadata); chunk indices along the leading axis
    start at ``start_chunk`` (appends)."""
    d = root / name
    d.mkdir(parents=True, exist_ok=True)
    vals = np.ascontiguousarray(var.values)
    dt = vals.dtype.newbyteorder("<") if vals.dtype.byteorder == ">" else vals.dtype
    vals = vals.astype(dt, copy=False)
    if dt.name not in _V3_TYPES:
        raise TypeError(f"cannot store dtype {vals.dtype} in a zarr array")
    chunks = _chunk_shape(var)
    for idx in _chunk_indices(vals.shape, chunks):
        sl = tuple(slice(i * c, (i + 1) * c) for i, c in zip(idx, chunks))
        block = np.zeros(chunks, dt)
        part = vals[sl]
        block[tuple(slice(0, n) for n in part.shape)] = part
        idx = (idx[0] + start_chunk, *idx[1:]) if idx else idx
        if fmt == 3:
            p = d.joinpath("c", *map(str, idx))
        else:
            p = d / (".".join(map(str, idx)) if idx else "0")
        p.parent.mkdir(parents=True, exist_ok=True)
        p.write_bytes(block.tobytes(order="C"))


def _array_meta(var: Variable, fmt: int, shape=None) -> dict:
    shape = list(shape if shape is not None else var.shape)
    dt = np.dtype(var.dtype).newbyteorder("<") if np.dtype(var.dtype).byteorder == ">" else np.dtype(var.dtype)
    fill = _json_fill(float("nan") if dt.kind == "f" else 0)
    if fmt == 3:
        return {"zarr_format": 3, "node_type": "array", "shape": shape, "data_type": _V3_TYPES[dt.name],
                "chunk_grid": {"name": "regular", "configuration": {"chunk_shape": list(_chunk_shape(var))}},
                "chunk_key_encoding": {"name": "default", "configuration": {"separator": "/"}},
                "fill_value": fill, "codecs": [{"name": "bytes", "configuration": {"endian": "little"}}],
                "attributes": dict(var.attrs), "dimension_names": list(var.dims)}
    return {"zarr_format": 2, "shape": shape, "chunks": list(_chunk_shape(var)), "dtype": dt.str,
            "compressor": None, "fill_value": fill, "order": "C", "filters": None, "dimension_separator": "."}


def save_dataset(ds: Dataset, path, *, mode: str = "w", zarr_format: int = 3) -> None:
    """Write a dataset to a zarr store (a directory).  ``mode``: "w" overwrite, "w-" fail if
    the store exists, "a" append along ``time`` (``append_to_dataset``) (``xarray.py:244-257``)."""
    path = Path(path)
    if mode == "a":
        return append_to_dataset(ds, path)
    if mode not in ("w", "w-"):
        raise ValueError(f"mode must be 'w', 'w-' or 'a', got {mode!r}")
    if path.exists():
        if mode == "w-":
            raise FileExistsError(f"zarr store {path} exists")
        shutil.rmtree(path)
    path.mkdir(parents=True)
    for name, var in ds.variables.items():
        _write_array(path, name, var, zarr_format)
        if zarr_format == 3:
            _write_json(path / name / "zarr.json", _array_meta(var, 3))
        else:
            _write_json(path / name / ".zarray", _array_meta(var, 2))
            _write_json(path / name / ".zattrs", {**var.attrs, "_ARRAY_DIMENSIONS": list(var.dims)})
    if zarr_format == 3:
        _write_json(path / "zarr.json", {"zarr_format": 3, "node_type": "group", "attributes": ds.attrs})
    else:
        _write_json(path / ".zgroup", {"zarr_format": 2})
        _write_json(path / ".zattrs", ds.attrs)


def _decode(raw: bytes, codecs: list, dtype: np.dtype, shape) -> np.ndarray:
    """One chunk's bytes through its codec chain, last codec first (zarr v3 names; the v2
    compressors are mapped onto them)."""
    endian = "little"
    for c in reversed(codecs):
        name = c["name"]
        if name == "gzip":
            raw = gzip.decompress(raw)
        elif name == "zlib":
            raw = zlib.decompress(raw)
        elif name == "zstd":
            try:
                import zstandard
            except ImportError as exc:
                raise RuntimeError("this store's chunks are zstd-compressed and the zstandard package is "
                                   "not installed") from exc
            raw = zstandard.ZstdDecompressor().decompressobj().decompress(raw)
        elif name == "bytes":
            endian = c.get("configuration", {}).get("endian", "little")
        elif name == "crc32c":
            raw = raw[:-4]
        else:
            raise RuntimeError(f"unsupported zarr codec {name!r}")
    dt = dtype.newbyteorder("<" if endian == "little" else ">")
    return np.frombuffer(raw, dt).astype(dtype).reshape(shape)


def _read_array(d: Path) -> Variable:
    if (d / "zarr.json").exists():
        m = json.loads((d / "zarr.json").read_text())
        dtype = np.dtype(m["data_type"])
        chunks = tuple(m["chunk_grid"]["configuration"]["chunk_shape"])
        enc = m.get("chunk_key_encoding", {"name": "default"})
        default = enc["name"] == "default"
        sep = enc.get("configuration", {}).get("separator", "/" if default else ".")
        prefix = ["c"] if default else []

        def key(idx):
            parts = prefix + [str(i) for i in idx]
            if not parts:
                return d / "0"
            return d.joinpath(*parts) if sep == "/" else d / sep.join(parts)

        codecs, dims, attrs = m.get("codecs", []), m.get("dimension_names"), dict(m.get("attributes", {}))
    else:
        m = json.loads((d / ".zarray").read_text())
        dt2 = np.dtype(m["dtype"])
        chunks = tuple(m["chunks"])
        sep = m.get("dimension_separator", ".")
        comp = m.get("compressor")
        codecs = [{"name": "bytes", "configuration": {"endian": "big" if dt2.byteorder == ">" else "little"}}]
        if comp is not None:
            if comp.get("id") not in ("gzip", "zlib", "zstd"):
                raise RuntimeError(f"unsupported zarr v2 compressor {comp!r}")
            codecs.append({"name": comp["id"]})
        dtype = dt2.newbyteorder("=")
        attrs = json.loads((d / ".zattrs").read_text()) if (d / ".zattrs").exists() else {}
        dims = attrs.pop("_ARRAY_DIMENSIONS", None)

        def key(idx):
            return d / (sep.join(str(i) for i in idx) if idx else "0")

    shape = tuple(m["shape"])
    out = np.empty(shape, dtype)
    out[...] = _parse_fill(m.get("fill_value"), dtype)
    for idx in _chunk_indices(shape, chunks):
        p = key(idx)
        if not p.exists():
            continue
        block = _decode(p.read_bytes(), codecs, dtype, chunks)
        sl = tuple(slice(i * c, min((i + 1) * c, n)) for i, c, n in zip(idx, chunks, shape))
        out[sl] = block[tuple(slice(0, s.stop - s.start) for s in sl)]
    if dims is None:
        dims = tuple(f"dim{i}" for i in range(len(shape)))
    return Variable(tuple(dims), out, attrs)


def load_dataset(path) -> Dataset:
    """Read a zarr store written by ``save_dataset`` (v3 or v2) into memory (``xarray.py:260-272``).
    One-dimensional variables named after their own dimension become coordinates."""
    path = Path(path)
    if (path / "zarr.json").exists():
        attrs = json.loads((path / "zarr.json").read_text()).get("attributes", {})
    elif (path / ".zgroup").exists():
        attrs = json.loads((path / ".zattrs").read_text()) if (path / ".zattrs").exists() else {}
    else:
        raise FileNotFoundError(f"{path} is not a zarr group")
    data_vars, coords = {}, {}
    for d in sorted(p for p in path.iterdir() if p.is_dir()):
        if not ((d / "zarr.json").exists() or (d / ".zarray").exists()):
            continue
        var = _read_array(d)
        (coords if var.dims == (d.name,) else data_vars)[d.name] = var
    return Dataset(data_vars, coords, attrs)


def append_to_dataset(ds: Dataset, path, *, append_dim: str = "time") -> None:
    """Append a dataset to an existing store along ``append_dim`` (``xarray.py:275-292``): every
    variable with that dimension gets the new slices (as new chunks), others must match."""
    path = Path(path)
    v3 = (path / "zarr.json").exists()
    old = load_dataset(path)
    for name, var in ds.variables.items():
        if name not in old:
            raise ValueError(f"variable {name!r} is not in the store {path}")
        have = old[name]
        if append_dim not in var.dims:
            if have.shape != var.shape:
                raise ValueError(f"variable {name!r} without {append_dim!r} changes shape")
            continue
        if var.dims != have.dims or var.dims[0] != append_dim:
            raise ValueError(f"variable {name!r}: dims {var.dims} do not extend {have.dims} along {append_dim!r}")
        if var.shape[1:] != have.shape[1:]:
            raise ValueError(f"variable {name!r}: shape {var.shape} does not extend {have.shape}")
        n0 = have.shape[0]
        merged = Variable(have.dims, np.zeros((0,) + have.shape[1:], have.dtype), have.attrs)
        _write_array(path, name, Variable(var.dims, var.values.astype(have.dtype), var.attrs), 3 if v3 else 2,
                     start_chunk=n0)
        shape = (n0 + var.shape[0],) + have.shape[1:]
        if v3:
            _write_json(path / name / "zarr.json", _array_meta(merged, 3, shape))
        else:
            _write_json(path / name / ".zarray", _array_meta(merged, 2, shape))


def save_state(state, path, *, time: float | None = None, attrs: dict | None = None) -> None:
    """``final_state.zarr``: one state written as the restart artifact (``cli/_run.py:357-364``)."""
    save_dataset(state_to_dataset(state, time=time, attrs=attrs), path, mode="w")


def load_state(path, state_class=None, *, time_index: int = -1, device=None):
    """A state read back from a restart or snapshot store (``cli/_run.py:840-862``)."""
    return dataset_to_state(load_dataset(path), state_class, time_index=time_index, device=device)


__all__: list[Any] = ["Dataset", "Variable", "state_to_dataset", "snapshots_to_dataset", "dataset_to_state",
                      "save_dataset", "load_dataset", "append_to_dataset", "save_state", "load_state"]
