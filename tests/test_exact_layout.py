"""The exact fill's memory accounting, on the host: ex_bytes leaves room for
every buffer ex_carve takes and for the largest scratch of the sorts and
scans in ex_run (tests/exact_layout_check.cu, compiled with nvcc and run
here; it launches nothing)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_exact_fill_buffers_fit_their_byte_count(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if not nvcc:
        pytest.skip("no nvcc")
    exe = str(tmp_path / "exact_layout_check")
    p = subprocess.run([nvcc, "-std=c++17", "--expt-relaxed-constexpr", "-gencode", "arch=compute_103a,code=sm_103a",
                        "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "lsdtt_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "exact_layout_check.cu"), "-o", exe],
                       capture_output=True, text=True)
    assert p.returncode == 0, p.stderr[-3000:]
    r = subprocess.run([exe], capture_output=True, text=True)
    print(r.stdout)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout + r.stderr
