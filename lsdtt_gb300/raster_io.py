"""Raster files without GDAL, for Python callers of the GPU path: ENVI
(.bil / .bsq / .img with an ENVI .hdr) and ESRI GridFloat (.flt with its
.hdr), read into and written from row-major float32 arrays (top row first)
with a nodata mask and the metadata the entry points take.

The same formats and rules as the C++ host layer (lsdtt_gb300/host/
raster_io.hpp), which tests/test_raster_io.py holds this module to; both
keep the conventions of the reference's GDAL loader (lsdtt_data_loader,
src/core/lsdtt_data_loader.hpp:395-560):
  * the metadata mirror lsdtt_raster_meta (src/core/lsdtt_raster_meta.hpp):
    x_min / y_min the left and bottom edges, square cells (non-square pixels
    are refused), no_data_value, the CRS as WKT where the header has one;
  * a pixel equal to no_data_value or not finite is nodata: mask 0, value
    no_data_value (lsdtt_data_loader.cpp:725-745).
"""
from __future__ import annotations

import dataclasses
import os
import re
from typing import Tuple

import numpy as np

__all__ = ["RasterMeta", "read_raster", "write_raster"]

# ENVI data type codes -> numpy sample types (byte order applied on read)
_ENVI_TYPES = {1: "u1", 2: "i2", 3: "i4", 4: "f4", 5: "f8", 12: "u2", 13: "u4"}


@dataclasses.dataclass
class RasterMeta:
    n_rows: int
    n_cols: int
    x_min: float = 0.0
    y_min: float = 0.0
    cell_size: float = 1.0
    no_data_value: float = -9999.0
    crs_wkt: str = ""


def _header_path(data_path: str) -> str:
    base, ext = os.path.splitext(data_path)
    a = (base if ext else data_path) + ".hdr"
    return a if os.path.exists(a) else data_path + ".hdr"


def _square(dx: float, dy: float, path: str) -> None:
    if not (dx > 0 and dy > 0) or abs(dx - dy) > 1e-9 * max(dx, dy):
        raise ValueError(f"raster_io: {path} has non-square or invalid pixels ({dx} x {dy}); "
                         f"square cells are required")


def _apply_nodata(data: np.ndarray, nodata: float) -> Tuple[np.ndarray, np.ndarray]:
    nd = np.float32(nodata)
    bad = (data == nd) | ~np.isfinite(data)
    data = data.copy()
    data[bad] = nd
    return data, (~bad).astype(np.uint8)


def _envi_pairs(text: str):
    """key = value pairs of an ENVI header; braced values may span lines."""
    pairs = []
    lines = text.splitlines()[1:]
    k = None
    buf = ""
    depth = 0
    for line in lines:
        if depth > 0:
            buf += "\n" + line
        else:
            if "=" not in line:
                continue
            k, buf = line.split("=", 1)
            k = k.strip().lower()
        depth = buf.count("{") - buf.count("}")
        if depth <= 0:
            pairs.append((k, buf.strip()))
            depth = 0
    return dict(pairs)


def _braced(v: str) -> str:
    v = v.strip()
    if v.startswith("{"):
        v = v[1:]
    if v.endswith("}"):
        v = v[:-1]
    return v.strip()


def _read_envi(path: str, text: str):
    kv = _envi_pairs(text)
    try:
        n_cols, n_rows = int(kv["samples"]), int(kv["lines"])
        dtype = int(kv["data type"])
    except KeyError as e:
        raise ValueError(f"raster_io: ENVI header of {path} has no {e.args[0]!r}") from None
    if int(kv.get("bands", "1")) != 1:
        raise ValueError(f"raster_io: {path} has {kv['bands']} bands; one is supported")
    if dtype not in _ENVI_TYPES:
        raise ValueError(f"raster_io: unsupported ENVI data type {dtype}")
    order = ">" if int(kv.get("byte order", "0")) == 1 else "<"
    offset = int(kv.get("header offset", "0"))
    meta = RasterMeta(n_rows, n_cols)
    if "data ignore value" in kv:
        meta.no_data_value = float(kv["data ignore value"])
    if "coordinate system string" in kv:
        meta.crs_wkt = _braced(kv["coordinate system string"])
    dx = dy = 1.0
    ex = ny = 0.0
    rx = ry = 1.0
    if "map info" in kv:
        f = [t.strip() for t in re.split(r",(?![^{\[]*[}\]])", _braced(kv["map info"]))]
        if len(f) < 7:
            raise ValueError(f"raster_io: malformed 'map info' in the header of {path}")
        rx, ry, ex, ny, dx, dy = (float(t) for t in f[1:7])
    _square(dx, dy, path)
    meta.cell_size = dx
    meta.x_min = ex - (rx - 1.0) * dx
    meta.y_min = ny + (ry - 1.0) * dy - n_rows * dy
    n = n_rows * n_cols
    dt = np.dtype(order + _ENVI_TYPES[dtype])
    raw = np.fromfile(path, dtype=dt, count=n, offset=offset)
    if raw.size != n:
        raise ValueError(f"raster_io: {path} is shorter than its header says")
    return raw.astype(np.float32).reshape(n_rows, n_cols), meta


def _read_gridfloat(path: str, text: str):
    kv = {}
    for line in text.splitlines():
        t = line.split()
        if len(t) >= 2:
            kv[t[0].lower()] = t[1]
    try:
        meta = RasterMeta(int(kv["nrows"]), int(kv["ncols"]))
        xk = "xllcorner" if "xllcorner" in kv else "xllcenter"
        yk = "yllcorner" if "yllcorner" in kv else "yllcenter"
        xll, yll = float(kv[xk]), float(kv[yk])
    except KeyError:
        raise ValueError(f"raster_io: the header of {path} lacks ncols, nrows or the corner") from None
    meta.cell_size = float(kv.get("cellsize", "1"))
    _square(meta.cell_size, meta.cell_size, path)
    meta.no_data_value = float(kv.get("nodata_value", "-9999"))
    meta.x_min = xll - 0.5 * meta.cell_size if xk == "xllcenter" else xll
    meta.y_min = yll - 0.5 * meta.cell_size if yk == "yllcenter" else yll
    order = ">" if kv.get("byteorder", "lsbfirst").lower() == "msbfirst" else "<"
    n = meta.n_rows * meta.n_cols
    raw = np.fromfile(path, dtype=np.dtype(order + "f4"), count=n)
    if raw.size != n:
        raise ValueError(f"raster_io: {path} is shorter than its header says")
    return raw.astype(np.float32).reshape(meta.n_rows, meta.n_cols), meta


def read_raster(path: str) -> Tuple[np.ndarray, np.ndarray, RasterMeta]:
    """(data float32 [n_rows, n_cols] top row first, mask uint8, meta)."""
    hp = _header_path(path)
    if not os.path.exists(hp):
        raise ValueError(f"raster_io: no header for {path} (looked for {hp})")
    text = open(hp).read()
    first = text.split("\n", 1)[0].strip().lower()
    data, meta = (_read_envi if first == "envi" else _read_gridfloat)(path, text)
    data, mask = _apply_nodata(data, meta.no_data_value)
    return data, mask, meta


def _fmt(v: float) -> str:
    return repr(float(v))


def write_raster(path: str, data: np.ndarray, meta: RasterMeta, fmt: str = "envi") -> None:
    """Write float32 little-endian samples to `path` and its header next to
    it (name.hdr): fmt "envi" (ENVI, bil) or "esri" (GridFloat)."""
    data = np.ascontiguousarray(data, dtype="<f4")
    if not (meta.n_rows > 0 and meta.n_cols > 0 and meta.cell_size > 0):
        raise ValueError("raster_io: invalid raster metadata")
    if data.shape != (meta.n_rows, meta.n_cols):
        raise ValueError(f"raster_io: a {data.shape} array for a {meta.n_rows} x {meta.n_cols} raster")
    base, ext = os.path.splitext(path)
    hp = (base if ext else path) + ".hdr"
    if fmt == "envi":
        y_max = meta.y_min + meta.n_rows * meta.cell_size
        h = (f"ENVI\nsamples = {meta.n_cols}\nlines = {meta.n_rows}\nbands = 1\nheader offset = 0\n"
             f"data type = 4\ninterleave = bil\nbyte order = 0\n"
             f"map info = {{Arbitrary, 1, 1, {_fmt(meta.x_min)}, {_fmt(y_max)}, {_fmt(meta.cell_size)}, "
             f"{_fmt(meta.cell_size)}}}\ndata ignore value = {_fmt(meta.no_data_value)}\n")
        if meta.crs_wkt:
            h += f"coordinate system string = {{{meta.crs_wkt}}}\n"
    elif fmt == "esri":
        h = (f"ncols {meta.n_cols}\nnrows {meta.n_rows}\nxllcorner {_fmt(meta.x_min)}\n"
             f"yllcorner {_fmt(meta.y_min)}\ncellsize {_fmt(meta.cell_size)}\n"
             f"NODATA_value {_fmt(meta.no_data_value)}\nbyteorder LSBFIRST\n")
    else:
        raise ValueError(f"raster_io: unknown format {fmt!r} (envi or esri)")
    with open(hp, "w") as f:
        f.write(h)
    data.tofile(path)
