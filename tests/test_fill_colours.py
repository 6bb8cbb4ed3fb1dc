"""The tile colouring that makes the fill deterministic, checked on the host
from the kernels' own header (lsdtt_gb300/csrc/fill_tile.cuh): for every
tile grid up to 11 x 11 tiles, with and without periodic axes, no two
distinct tiles that are neighbours (8-neighbourhood, wrapping on periodic
axes) share a colour, and fill_colour_mask has the bit of every colour in
use. A fill pass relaxes one colour at a time in place, so this is what lets
every tile read settled or untouched neighbours only."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <cstdio>
#include "fill_tile.cuh"
using namespace lsdtt_gb300;
int main()
{
    long checked = 0;
    for (int ntx = 1; ntx <= 11; ++ntx)
        for (int nty = 1; nty <= 11; ++nty)
            for (int p = 0; p < 4; ++p)
            {
                const bool per_ns = p & 1, per_ew = p & 2;
                const unsigned mask = fill_colour_mask(ntx, nty, per_ns, per_ew);
                for (int ty = 0; ty < nty; ++ty)
                    for (int tx = 0; tx < ntx; ++tx)
                    {
                        const int c = fill_colour(tx, ty, ntx, nty, per_ns, per_ew);
                        if (c < 0 || c >= kFillColours || !((mask >> c) & 1u))
                        {
                            std::printf("FAIL colour %d of tile (%d,%d) in %dx%d p=%d mask %x\n", c, tx, ty, ntx,
                                        nty, p, mask);
                            return 1;
                        }
                        for (int dy = -1; dy <= 1; ++dy)
                            for (int dx = -1; dx <= 1; ++dx)
                            {
                                int yy = ty + dy, xx = tx + dx;
                                if (per_ns) yy = (yy + nty) % nty;
                                if (per_ew) xx = (xx + ntx) % ntx;
                                if (yy < 0 || yy >= nty || xx < 0 || xx >= ntx) continue;
                                if (yy == ty && xx == tx) continue;
                                ++checked;
                                if (fill_colour(xx, yy, ntx, nty, per_ns, per_ew) == c)
                                {
                                    std::printf("FAIL tiles (%d,%d) and (%d,%d) share colour %d in %dx%d p=%d\n", tx,
                                                ty, xx, yy, c, ntx, nty, p);
                                    return 1;
                                }
                            }
                    }
            }
    std::printf("OK %ld\n", checked);
    return 0;
}
"""


def test_no_two_neighbouring_tiles_share_a_colour(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not found")
    src = tmp_path / "colours.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "colours"
    subprocess.run([nvcc, "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a", "-I",
                    os.path.join(ROOT, "lsdtt_gb300", "csrc"), str(src), "-o", str(exe)], check=True,
                   capture_output=True, timeout=300)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0 and out.stdout.startswith("OK"), out.stdout
