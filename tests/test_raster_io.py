"""The GDAL-free raster I/O of the host layer (lsdtt_gb300/host/raster_io.hpp)
through its command-line driver tests/raster_io_check.cpp, compiled here
with g++, and its Python counterpart (lsdtt_gb300/raster_io.py), held to
it: round trips through both formats they write (ENVI .bil and ESRI
GridFloat), headers written by hand in the ways other tools write them
(big-endian float64 and int16 ENVI bands, a header offset, a reference pixel
other than the first, a CRS string over several lines, cell-centre corners,
MSBFIRST GridFloat), the reference loader's nodata rule (a pixel equal to
the sentinel or not finite gets mask 0 and the sentinel as its value:
lsdtt_data_loader.cpp:725-745) and the refusals (non-square pixels, a
missing header, a short data file)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def rio(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    exe = str(tmp_path_factory.mktemp("rio") / "raster_io_check")
    p = subprocess.run([gxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", ROOT,
                        os.path.join(ROOT, "tests", "raster_io_check.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert p.returncode == 0, p.stderr[-3000:]
    return exe


def _read(rio, path, tmp):
    pre = str(tmp / "out")
    p = subprocess.run([rio, "read", str(path), pre], capture_output=True, text=True)
    if p.returncode != 0:
        return None, None, None, p
    first, wkt = open(pre + ".meta").read().split("\n", 1)
    f = first.split()
    meta = dict(n_rows=int(f[0]), n_cols=int(f[1]), x_min=float(f[2]), y_min=float(f[3]), cell_size=float(f[4]),
                no_data_value=float(f[5]), crs_wkt=wkt[:-1] if wkt.endswith("\n") else wkt)
    data = np.fromfile(pre + ".data", np.float32).reshape(meta["n_rows"], meta["n_cols"])
    mask = np.fromfile(pre + ".mask", np.uint8).reshape(meta["n_rows"], meta["n_cols"])
    return data, mask, meta, p


def _write(rio, values, path, x_min, y_min, cell, nodata, fmt, tmp, wkt=None):
    raw = str(tmp / "values.f32")
    np.ascontiguousarray(values, np.float32).tofile(raw)
    cmd = [rio, "write", raw, str(values.shape[0]), str(values.shape[1]), repr(x_min), repr(y_min), repr(cell),
           repr(nodata), fmt, str(path)]
    if wkt is not None:
        cmd.append(wkt)
    return subprocess.run(cmd, capture_output=True, text=True)


def _expected(values, nodata):
    """The reference loader's rule: the sentinel or a non-finite value is
    nodata (mask 0) and holds the sentinel."""
    v = np.asarray(values, np.float32).copy()
    bad = (v == np.float32(nodata)) | ~np.isfinite(v)
    v[bad] = np.float32(nodata)
    return v, (~bad).astype(np.uint8)


def _surface(rows, cols, seed):
    rng = np.random.default_rng(seed)
    z = (rng.random((rows, cols)) * 100.0).astype(np.float32)
    z[0, :3] = np.nan
    z[rows // 2, cols // 2] = np.inf
    z[-1, -1] = -9999.0
    return z


@pytest.mark.parametrize("fmt,name", [("envi", "dem.bil"), ("esri", "dem.flt")])
def test_round_trip(rio, tmp_path, fmt, name):
    z = _surface(37, 53, 1)
    wkt = 'PROJCS["WGS 84 / UTM zone 30N",GEOGCS["WGS 84"]]' if fmt == "envi" else None
    p = _write(rio, z, tmp_path / name, 412345.5, 6012340.25, 10.0, -9999.0, fmt, tmp_path, wkt)
    assert p.returncode == 0, p.stderr
    data, mask, meta, p = _read(rio, tmp_path / name, tmp_path)
    assert p.returncode == 0, p.stderr
    want, wmask = _expected(z, -9999.0)
    assert np.array_equal(data.view(np.uint32), want.view(np.uint32))
    assert np.array_equal(mask, wmask)
    assert (meta["n_rows"], meta["n_cols"]) == z.shape
    assert meta["x_min"] == 412345.5 and meta["y_min"] == 6012340.25 and meta["cell_size"] == 10.0
    assert meta["no_data_value"] == -9999.0
    assert meta["crs_wkt"] == (wkt or "")


def test_envi_written_elsewhere(rio, tmp_path):
    """A big-endian float64 band after a 16-byte header offset, the map
    info's reference pixel at (2, 3), the nodata value and a CRS string over
    several lines."""
    rows, cols, cell = 11, 7, 30.0
    z = _surface(rows, cols, 2).astype(np.float64)
    open(tmp_path / "e.bsq", "wb").write(b"\0" * 16 + z.astype(">f8").tobytes())
    east, north = 500030.0, 4200000.0  # upper-left corner of pixel (2, 3), 1-based
    open(tmp_path / "e.hdr", "w").write(
        "ENVI\ndescription = {\n  a DEM written by\n  another tool}\nsamples = 7\nlines   = 11\nbands = 1\n"
        "header offset = 16\nfile type = ENVI Standard\ndata type = 5\ninterleave = bsq\nbyte order = 1\n"
        f"map info = {{UTM, 2.000, 3.000, {east}, {north}, {cell}, {cell}, 30, North, WGS-84, units=Meters}}\n"
        "coordinate system string = {PROJCS[\"UTM 30N\",\n GEOGCS[\"WGS 84\"]]}\n"
        "data ignore value = -9999\n")
    data, mask, meta, p = _read(rio, tmp_path / "e.bsq", tmp_path)
    assert p.returncode == 0, p.stderr
    want, wmask = _expected(z.astype(np.float32), -9999.0)
    assert np.array_equal(data.view(np.uint32), want.view(np.uint32))
    assert np.array_equal(mask, wmask)
    assert meta["x_min"] == east - 1 * cell
    assert meta["y_min"] == (north + 2 * cell) - rows * cell
    assert meta["cell_size"] == cell
    assert meta["crs_wkt"] == 'PROJCS["UTM 30N",\n GEOGCS["WGS 84"]]'


def test_envi_int16_band(rio, tmp_path):
    z = np.arange(-30, 30, dtype=np.int16).reshape(6, 10)
    z[2, 3] = -32768
    open(tmp_path / "i.bil", "wb").write(z.astype("<i2").tobytes())
    open(tmp_path / "i.hdr", "w").write(
        "ENVI\nsamples = 10\nlines = 6\nbands = 1\nheader offset = 0\ndata type = 2\ninterleave = bil\n"
        "byte order = 0\nmap info = {Arbitrary, 1, 1, 0, 60, 10, 10}\ndata ignore value = -32768\n")
    data, mask, meta, p = _read(rio, tmp_path / "i.bil", tmp_path)
    assert p.returncode == 0, p.stderr
    want, wmask = _expected(z.astype(np.float32), -32768.0)
    assert np.array_equal(data, want) and np.array_equal(mask, wmask)
    assert (meta["x_min"], meta["y_min"], meta["cell_size"]) == (0.0, 0.0, 10.0)


def test_gridfloat_cell_centres_and_msbfirst(rio, tmp_path):
    z = _surface(9, 12, 3)
    z.astype(">f4").tofile(tmp_path / "g.flt")
    open(tmp_path / "g.hdr", "w").write("ncols 12\nnrows 9\nxllcenter 105.0\nyllcenter 205.0\ncellsize 10\n"
                                        "NODATA_value -9999\nbyteorder MSBFIRST\n")
    data, mask, meta, p = _read(rio, tmp_path / "g.flt", tmp_path)
    assert p.returncode == 0, p.stderr
    want, wmask = _expected(z, -9999.0)
    assert np.array_equal(data.view(np.uint32), want.view(np.uint32)) and np.array_equal(mask, wmask)
    assert (meta["x_min"], meta["y_min"]) == (100.0, 200.0)


def test_refusals(rio, tmp_path):
    # non-square pixels (the reference's loader refuses them too)
    np.zeros((4, 4), "<f4").tofile(tmp_path / "n.bil")
    open(tmp_path / "n.hdr", "w").write("ENVI\nsamples = 4\nlines = 4\nbands = 1\ndata type = 4\n"
                                        "byte order = 0\nmap info = {Arbitrary, 1, 1, 0, 40, 10, 20}\n")
    _, _, _, p = _read(rio, tmp_path / "n.bil", tmp_path)
    assert p.returncode == 3 and "non-square" in p.stderr
    # no header
    np.zeros((4, 4), "<f4").tofile(tmp_path / "lonely.flt")
    _, _, _, p = _read(rio, tmp_path / "lonely.flt", tmp_path)
    assert p.returncode == 3 and "no header" in p.stderr
    # data shorter than the header says
    np.zeros((3, 4), "<f4").tofile(tmp_path / "s.flt")
    open(tmp_path / "s.hdr", "w").write("ncols 4\nnrows 4\nxllcorner 0\nyllcorner 0\ncellsize 1\n")
    _, _, _, p = _read(rio, tmp_path / "s.flt", tmp_path)
    assert p.returncode == 3 and "shorter" in p.stderr


def _same(py, cpp):
    """The Python module's (data, mask, RasterMeta) equals the C++ driver's
    (data, mask, meta dict)."""
    da, ma, mta = py
    db, mb, mtb = cpp
    assert np.array_equal(da.view(np.uint32), db.view(np.uint32))
    assert np.array_equal(ma, mb)
    for k in ("n_rows", "n_cols", "x_min", "y_min", "cell_size", "no_data_value", "crs_wkt"):
        assert getattr(mta, k) == mtb[k], k


def test_python_module_matches_the_cpp_header(rio, tmp_path):
    """lsdtt_gb300.raster_io (numpy) and host/raster_io.hpp read every file
    of the tests above alike, and each reads what the other writes."""
    from lsdtt_gb300 import raster_io as R
    z = _surface(23, 31, 4)
    wkt = 'PROJCS["x",GEOGCS["y"]]'
    # C++ writes, Python reads
    for fmt, name in (("envi", "c.bil"), ("esri", "c.flt")):
        p = _write(rio, z, tmp_path / name, 1000.5, 2000.25, 5.0, -9999.0, fmt, tmp_path,
                   wkt if fmt == "envi" else None)
        assert p.returncode == 0, p.stderr
        data, mask, meta, p = _read(rio, tmp_path / name, tmp_path)
        py = R.read_raster(str(tmp_path / name))
        _same(py, (data, mask, meta))
    # Python writes, C++ reads
    for fmt, name in (("envi", "p.bil"), ("esri", "p.flt")):
        m = R.RasterMeta(23, 31, 1000.5, 2000.25, 5.0, -9999.0, wkt if fmt == "envi" else "")
        R.write_raster(str(tmp_path / name), z, m, fmt)
        data, mask, meta, p = _read(rio, tmp_path / name, tmp_path)
        assert p.returncode == 0, p.stderr
        _same(R.read_raster(str(tmp_path / name)), (data, mask, meta))
        want, wmask = _expected(z, -9999.0)
        assert np.array_equal(data.view(np.uint32), want.view(np.uint32)) and np.array_equal(mask, wmask)
        assert (meta["x_min"], meta["y_min"], meta["cell_size"], meta["crs_wkt"]) == (1000.5, 2000.25, 5.0, m.crs_wkt)
    # a foreign ENVI header: big-endian float64 after an offset, reference pixel (2, 3), CRS over two lines
    zz = _surface(11, 7, 2).astype(np.float64)
    open(tmp_path / "e.bsq", "wb").write(b"\0" * 16 + zz.astype(">f8").tobytes())
    open(tmp_path / "e.hdr", "w").write(
        "ENVI\nsamples = 7\nlines = 11\nbands = 1\nheader offset = 16\ndata type = 5\nbyte order = 1\n"
        "map info = {UTM, 2, 3, 500030.0, 4200000.0, 30.0, 30.0, 30, North}\n"
        "coordinate system string = {PROJCS[\"a\",\n GEOGCS[\"b\"]]}\ndata ignore value = -9999\n")
    data, mask, meta, p = _read(rio, tmp_path / "e.bsq", tmp_path)
    _same(R.read_raster(str(tmp_path / "e.bsq")), (data, mask, meta))
    # refusals
    np.zeros((4, 4), "<f4").tofile(tmp_path / "n.bil")
    open(tmp_path / "n.hdr", "w").write("ENVI\nsamples = 4\nlines = 4\nbands = 1\ndata type = 4\n"
                                        "map info = {Arbitrary, 1, 1, 0, 40, 10, 20}\n")
    with pytest.raises(ValueError, match="non-square"):
        R.read_raster(str(tmp_path / "n.bil"))
    np.zeros((3, 4), "<f4").tofile(tmp_path / "s.flt")
    open(tmp_path / "s.hdr", "w").write("ncols 4\nnrows 4\nxllcorner 0\nyllcorner 0\ncellsize 1\n")
    with pytest.raises(ValueError, match="shorter"):
        R.read_raster(str(tmp_path / "s.flt"))
