"""Writes tests/golden/roering_512.npz: a 512 x 512 Roering (nonlinear)
implicit hillslope step computed by the FP64 restatement of the reference's
Newton + sparse LU solve (oracle/hillslope.py: compute_hillslope_newton /
_transient, newton_cpu.cpp:196-788 on the operator of
hillslope_operator_cpu.hpp:83-322). The restatement takes about a minute at
this size, so the GPU test compares against these stored vectors instead of
re-running it; the input surface is stored too (numpy's FFT is not
guaranteed to give the same bits on every platform).

    python tests/golden/make_roering_fixture.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import hillslope as H  # noqa: E402
from tests import surfaces  # noqa: E402

CASE = dict(cell=5.0, bc="nnon", D=0.01, Sc=1.0, dt=2.5e4, relief=30.0, seed=21, shape=(512, 512))


def main():
    nr, nc = CASE["shape"]
    z = surfaces.fractal(nr, nc, CASE["relief"], CASE["seed"])
    m = np.ones_like(z, np.uint8)
    out, n_sub, iters = H.transient(z, m, CASE["cell"], CASE["bc"], CASE["D"], CASE["Sc"], CASE["dt"])
    path = os.path.join(HERE, "roering_512.npz")
    np.savez_compressed(path, z=z, out=out, n_sub=n_sub, iters=iters,
                        **{k: np.asarray(v) for k, v in CASE.items() if k != "shape"})
    print(f"{path}: {n_sub} sub-steps, {iters} Newton iterations")


if __name__ == "__main__":
    main()
