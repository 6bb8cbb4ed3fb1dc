"""The C++ drop-in for lsdtt3's abstract D8 seam
(lsdtt_gb300/host/lsdtt_flowinfo_gpu.hpp) compiles against the reference's
own headers and implements every pure virtual of lsdtt_flow_base (it is not
abstract), and the GPU overloads at the fill, stream-power and LEM seams
(lsdtt_gb300/host/lsdtt_gpu_overloads.hpp) resolve with the reference's own
argument lists. The same engine runs on the GPU in
tests/test_gpu_host_engine.py, which needs no checkout. Needs a reference checkout (LSDTT3_SRC or the default location);
skipped where there is none."""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "print-src"], capture_output=True,
                     text=True).stdout.strip()


@pytest.mark.skipif(not REF or not os.path.isdir(REF), reason="no lsdtt3 checkout")
def test_seam_compiles_and_is_concrete():
    gxx = shutil.which("g++")
    assert gxx
    src = """
#include "lsdtt_gb300/host/lsdtt_flowinfo_gpu.hpp"
#include <type_traits>
static_assert(!std::is_abstract<lsdtt::lsdtt_flowinfo_gpu>::value, "every pure virtual is implemented");
static_assert(std::is_base_of<lsdtt::lsdtt_flow_base, lsdtt::lsdtt_flowinfo_gpu>::value, "behind the seam");
std::unique_ptr<lsdtt::lsdtt_flow_base> make_gpu(const lsdtt::lsdtt_array2d_f& d, const lsdtt::lsdtt_array2d_u8& m,
                                                 const lsdtt::lsdtt_raster_meta& meta,
                                                 const lsdtt::lsdtt_flowinfo_options& o)
{ return std::make_unique<lsdtt::lsdtt_flowinfo_gpu>(d, m, meta, o); }
#include "lsdtt_gb300/host/lsdtt_gpu_overloads.hpp"
// The three overloads resolve with the reference's own argument lists.
lsdtt::lsdtt_raster_cpu sp(const lsdtt::lsdtt_raster_cpu& dem, const lsdtt::lsdtt_flowinfo_gpu& flow)
{ return lsdtt::compute_d8_stream_power_incision(dem, flow, 1e-5f, 0.5f, 1.0f, 1000.0f, 0.0f, true, 1e-5f); }
lsdtt::lsdtt_raster_cpu fill(const lsdtt::lsdtt_raster_cpu& r) { return lsdtt::fill_pits_gpu(r, 1e-4f, "nnon"); }
std::pair<lsdtt::lsdtt_raster_cpu, lsdtt::lsdtt_lem_step_stats> lem(const lsdtt::lsdtt_raster_cpu& dem,
                                                                   const lsdtt::lsdtt_lem_options& o,
                                                                   const std::vector<std::int64_t>& bf)
{ return lsdtt::run_lem_step_gpu(dem, o, bf); }
"""
    with tempfile.TemporaryDirectory() as td:
        f = os.path.join(td, "seam.cpp")
        open(f, "w").write(src)
        cmd = [gxx, "-std=c++17", "-c", f, "-o", os.path.join(td, "seam.o"), "-I", ROOT,
               "-I", os.path.join(ROOT, "include"), "-I", os.path.join(REF, "core"), "-I", os.path.join(REF, "utils"),
               "-I", os.path.join(REF, "cpu"), "-I", "/usr/local/cuda/include"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        assert p.returncode == 0, p.stderr[-3000:]
