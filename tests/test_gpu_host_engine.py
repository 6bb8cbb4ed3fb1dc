"""The C++ host layer (lsdtt_gb300/host/gb300_engine.hpp) run on the GPU:
a small C++ program (tests/host_engine_check.cpp) is compiled against it and
the C ABI, run on a surface, and every output it writes is compared with the
oracle: the epsilon fill against the GPU fill (the same kernels, bit for
bit), every D8 component and both accumulations bit for bit against
lsdtt_flowinfo, upslope_nodes slices against the oracle's s-vector, stream
power bit for bit against compute_d8_stream_power_incision, the LEM step
against the Python path of the same library, and the exception types and
messages the reference throws."""
import glob
import os
import shutil
import subprocess

import numpy as np
import pytest

from tests import surfaces

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _compile(tmp):
    gxx = shutil.which("g++")
    assert gxx, "g++ is needed to build the C++ check"
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    libdir = os.path.join(ROOT, "lsdtt_gb300")
    exe = os.path.join(tmp, "host_engine_check")
    libs = ["-L", libdir, "-llsdtt_gb300", f"-Wl,-rpath,{libdir}"]
    for d in [os.path.join(cuda, "lib64")] + glob.glob(os.path.join(cuda, "targets", "*", "lib")):
        libs += ["-L", d, f"-Wl,-rpath,{d}"]
    cmd = [gxx, "-std=c++17", "-O2", os.path.join(ROOT, "tests", "host_engine_check.cpp"), "-o", exe,
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "lsdtt_gb300", "host"),
           "-I", os.path.join(cuda, "include"), *libs, "-lcudart"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr[-3000:]
    return exe


@pytest.mark.parametrize("case", ["noise_tilt_nnon", "fractal_popo"])
def test_host_engine_against_oracle(port, tmp_path, case):
    import lsdtt_gb300 as G
    if case == "noise_tilt_nnon":
        z = port.noise_tilt_surface(200, 260, 30.0, 5, 0.0, 1.0, "nnon", 0.001)
        cell, bc, K, m_exp, n_exp = 30.0, "nnon", 1e-5, 0.5, 1.0
    else:
        z = surfaces.add_pits(surfaces.fractal(192, 224, 200.0, 8), 40, 8)
        cell, bc, K, m_exp, n_exp = 10.0, "popo", 2e-5, 0.45, 1.5
    mask = np.ones_like(z, np.uint8)
    dt, U, D, eps = 1000.0, 1e-3, 0.01, 1e-4
    f = port.fill_pits(z, mask, cell, bc, eps)
    w = np.random.default_rng(3).uniform(0.5, 2.0, z.size)
    d = str(tmp_path)
    z.astype(np.float32).tofile(os.path.join(d, "z.f32"))
    f.astype(np.float32).tofile(os.path.join(d, "f.f32"))
    mask.tofile(os.path.join(d, "mask.u8"))
    w.tofile(os.path.join(d, "w.f64"))
    with open(os.path.join(d, "meta.txt"), "w") as fh:
        fh.write(f"{z.shape[0]} {z.shape[1]} {cell!r} {bc} {eps!r} {K!r} {m_exp!r} {n_exp!r} {dt!r} {U!r} {D!r}\n")
    exe = _compile(d)
    p = subprocess.run([exe, d], capture_output=True, text=True)
    assert p.returncode == 0, p.stderr

    def rd(name, dt_):
        return np.fromfile(os.path.join(d, name), dtype=dt_)

    gf = G.fill_pits(z, mask, cell, bc, eps).cpu().numpy().ravel()
    assert np.array_equal(rd("filled.f32", np.float32).view(np.uint32), gf.view(np.uint32))

    want = port.flowinfo(f, mask, cell, bc, allow_pits_as_outlets=True)
    want_w = port.flowinfo(f, mask, cell, bc, allow_pits_as_outlets=True, weights=w)
    assert np.array_equal(rd("receiver.i64", np.int64), want["receiver"])
    assert np.array_equal(rd("direction.u8", np.uint8), want["direction"])
    assert np.array_equal(rd("donors.u8", np.uint8), want["donors"])
    assert np.array_equal(rd("outlets.i64", np.int64), want["outlets"])
    assert np.array_equal(rd("topo.i64", np.int64), want["topo"])
    assert np.array_equal(rd("svec.i64", np.int64), want["s_vector"])
    assert np.array_equal(rd("start.i64", np.int64), want["sv_start"])
    assert np.array_equal(rd("size.u64", np.uint64), want["sv_size"])
    assert np.array_equal(rd("area.f64", np.float64).view(np.uint64), want["accum"].view(np.uint64))
    assert np.array_equal(rd("weighted.f64", np.float64).view(np.uint64), want_w["accum"].view(np.uint64))

    ups = rd("upslope.i64", np.int64)
    i, checked = 0, 0
    while i < ups.size:
        c, k = int(ups[i]), int(ups[i + 1])
        s0 = int(want["sv_start"][c])
        assert np.array_equal(ups[i + 2:i + 2 + k], want["s_vector"][s0:s0 + k]), c
        i += 2 + k
        checked += 1
    assert checked > 100

    qd = port.flow_query("distance_from_outlet", f, mask, cell, bc)
    assert np.array_equal(rd("q_dist.f32", np.float32).view(np.uint32), qd[0].ravel().view(np.uint32))
    assert np.array_equal(rd("q_dist_mask.u8", np.uint8), qd[1].ravel())
    qs = port.flow_query("upslope_sum", f, mask, cell, bc, values=w.reshape(z.shape).astype(np.float32),
                         vmask=mask, include_self=True)
    assert np.array_equal(rd("q_upsum.f32", np.float32).view(np.uint32), qs[0].ravel().view(np.uint32))

    sp = port.stream_power(f, mask, cell, bc, K, m_exp, n_exp, dt)
    assert np.array_equal(rd("sp.f32", np.float32).view(np.uint32), sp.ravel().view(np.uint32))

    model = G.LandscapeModel(f, mask, cell, bc, timestep=dt, erodibility=K, m_exponent=m_exp, n_exponent=n_exp,
                             uplift_rate=U, hillslope_diffusivity=D, fill_min_slope=0.0)
    model.step()
    lem = rd("lem.f32", np.float32)
    assert np.array_equal(lem.view(np.uint32), model.z.cpu().numpy().ravel().view(np.uint32))
    model.close()

    errs = open(os.path.join(d, "errors.txt")).read().splitlines()
    assert errs[0].startswith("out_of_range lsdtt_flowinfo: flat index out of range")
    assert errs[1].startswith("runtime_error 4 lsdtt_flowinfo: could not assign a receiver at row"), errs[1]
    assert errs[2] == (f"invalid_argument lsdtt_flowinfo: forced outlet flat index {z.size + 5} (entry 0) is "
                       f"outside the raster, which has {z.size} cells"), errs[2]
