"""The FP64 hillslope restatement against the reference's own analytic
checks (tests/cpp/test_hillslope_implicit.cpp volume conservation under
no-flux boundaries; test_hillslope_newton.cpp Dirichlet cells held; linear
problems converge in one Newton step)."""
import numpy as np

import oracle.hillslope as H
from tests import surfaces


def test_noflux_conserves_volume():
    z = surfaces.fractal(48, 40, 30.0, 3)
    m = np.ones_like(z, np.uint8)
    zn, it, F = H.linear_step(z, m, 5.0, "nnnn", 0.05, 500.0)
    assert it == 1 and F < 1e-12
    assert abs(zn.astype(np.float64).sum() - z.astype(np.float64).sum()) < 1e-6 * z.size
    assert np.abs(zn - z).max() > 1e-4  # the step did something


def test_dirichlet_edges_are_held():
    z = surfaces.fractal(32, 32, 30.0, 4)
    m = np.ones_like(z, np.uint8)
    zn, _, _ = H.linear_step(z, m, 5.0, "oooo", 0.05, 500.0)
    for edge in (zn[0], zn[-1], zn[:, 0], zn[:, -1]):
        pass
    assert np.array_equal(zn[0], z[0]) and np.array_equal(zn[-1], z[-1])
    assert np.array_equal(zn[:, 0], z[:, 0]) and np.array_equal(zn[:, -1], z[:, -1])


def test_masked_cells_untouched_and_periodic_wrap():
    rng = np.random.default_rng(1)
    z = surfaces.fractal(30, 36, 10.0, 5)
    m = (rng.random(z.shape) > 0.1).astype(np.uint8)
    zn, _, _ = H.linear_step(z, m, 5.0, "popo", 0.05, 500.0)
    assert np.array_equal(zn[m == 0], z[m == 0])


def test_roering_newton_fails_at_the_minimum_substep_beyond_sc():
    """The reference's Roering Newton (hillslope_newton_cpu.cpp: the line
    search that keeps the field feasible, :578-632, and the sub-step
    controller, :750-768) on a field where most cells are steeper than Sc:
    no step size reduces the residual, and the transient solve stops with
    "Newton failed at the minimum sub-step" (the reference's message then
    asks for its damped-Picard solver). The same surface below Sc converges.
    This is why the Roering workloads run with relief scaled under Sc."""
    import pytest
    z = surfaces.fractal(48, 48, 1.0, 3).astype(np.float64)
    z = (z - z.min()) / (z.max() - z.min())
    m = np.ones(z.shape, np.uint8)
    cell, D, Sc, dt = 5.0, 0.01, 1.0, 1000.0
    steep = (z * 120.0).astype(np.float32)
    gy, gx = np.gradient(steep.astype(np.float64), cell)
    assert np.mean(np.hypot(gx, gy) > Sc) > 0.8
    with pytest.raises(RuntimeError, match="minimum sub-step"):
        H.transient(steep, m, cell, "oooo", D, Sc, dt, True)
    gentle = (z * 5.0).astype(np.float32)
    out, n_sub, iters = H.transient(gentle, m, cell, "oooo", D, Sc, dt, True)
    assert n_sub >= 1 and np.all(np.isfinite(out))
