"""The GPU's epsilon-fill method, restated on the CPU (tests/window_model.cpp,
compiled here with g++): value windows cut at epsilon-0 pour levels,
chained from the lowest cut, each replayed by the sequential rules (the
one-warp replay) or one FIFO sweep at a time with pop times as a fixed point
(the block replay). Both chains give the oracle's priority flood with
(row, col) heap ties bit for bit, and the two replays agree window by window,
on the surfaces the GPU tests use (a noise-plus-tilt surface, one long
episode; pitted fractals, many short ones; periodic axes; a filled surface
with fresh erosion pits; interior nodata holes)."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from tests import surfaces

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def model(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    so = str(tmp_path_factory.mktemp("wm") / "libwindow_model.so")
    p = subprocess.run([gxx, "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-shared", "-fPIC",
                        os.path.join(ROOT, "tests", "window_model.cpp"), "-o", so], capture_output=True, text=True)
    assert p.returncode == 0, p.stderr[-3000:]
    lib = ctypes.CDLL(so)
    f = lib.window_model_fill
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                  ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    return f


def _fill(model, z, m, bc, cell, eps, mode):
    z = np.ascontiguousarray(z, np.float32)
    m = np.ascontiguousarray(m, np.uint8)
    out = np.empty_like(z)
    st = np.zeros(5, np.int64)
    per_ns = bc[0] in "pP"
    per_ew = bc[1] in "pP"
    rc = model(z.ctypes.data, m.ctypes.data, z.shape[0], z.shape[1], int(per_ns), int(per_ew), cell, eps, mode,
               out.ctypes.data, st.ctypes.data)
    assert rc == 0, rc
    return out, st


def _cases(port):
    one = lambda z: np.ones_like(z, np.uint8)  # noqa: E731
    z1 = port.noise_tilt_surface(96, 128, 30.0, 3, 0.0, 1.0, "nnon", 0.001)
    z2 = surfaces.fractal_pits(96, seed=5)
    z3 = surfaces.add_pits(surfaces.fractal(40, 56, 150.0, 8), 12, 4)
    z4 = port.fill_pits(z1, one(z1), 30.0, "nnon", 1e-4)
    rng = np.random.default_rng(21)
    z4 = (z4 - (rng.random(z4.shape) < 0.08) * rng.random(z4.shape).astype(np.float32) * 0.02).astype(np.float32)
    z5 = surfaces.fractal_pits(80, seed=9)
    m5 = one(z5)
    m5[20:31, 10:27] = 0
    m5[50:53, 40:66] = 0
    return [("noise_tilt_96x128", z1, one(z1), "nnon", 30.0, 1e-4),
            ("fractal_pits_96", z2, one(z2), "oooo", 10.0, 1e-4),
            ("fractal_popo_40x56", z3, one(z3), "popo", 10.0, 1e-4),
            ("fractal_opop_40x56", z3, one(z3), "opop", 10.0, 1e-3),
            ("lem_like_96x128", z4, one(z4), "nnon", 30.0, 1e-4),
            ("fractal_holes_80", z5, m5, "oooo", 10.0, 1e-4)]


def test_chained_windows_equal_the_priority_flood(model, port):
    for name, z, m, bc, cell, eps in _cases(port):
        want = port.fill_pits_index_ties(z, m, cell, bc, eps)
        got, st = _fill(model, z, m, bc, cell, eps, 0)
        v = m != 0
        nd = int((got[v].view(np.uint32) != want[v].view(np.uint32)).sum())
        print(f"{name}: {int(((want != z) & (m != 0)).sum())} raised cells, {st[0]} cuts, {st[1]} candidates, "
              f"{st[2]} windows on the chain; {nd} cells differ")
        assert nd == 0, name


def test_sweep_replays_equal_the_sequential_replays(model, port):
    for name, z, m, bc, cell, eps in _cases(port):
        want = port.fill_pits_index_ties(z, m, cell, bc, eps)
        got, st = _fill(model, z, m, bc, cell, eps, 2)
        assert st[3] == 0, (name, int(st[3]))
        sw, _ = _fill(model, z, m, bc, cell, eps, 1)
        print(f"{name}: {st[4]} sweeps over {st[2]} windows, every window alike")
        v = m != 0
        assert np.array_equal(sw[v].view(np.uint32), want[v].view(np.uint32)), name
