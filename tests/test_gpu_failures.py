"""Failure detection on the GPU path, in forms that fault, trap or hang no
GPU: every failure is made on the host side (an iteration cap, a poisoned
input, a network whose output is not finite) or by running the library's
own bounded waits against a condition nothing satisfies. Each case checks
the status the reference's behaviour corresponds to, and that the context
stays usable afterwards.

* non-convergence: the reference reports a hillslope solve that does not
  converge (lem_cpu.cpp:563-582); here the solve, the single-grid LEM step
  and the ensemble step return LSDTT_GPU_ENOCONV with a message;
* bounded waits: the cooperative sweep's grid barrier and the tensor-core
  convolutions' mbarrier wait give up and report LSDTT_GPU_ETIMEOUT;
* PCG breakdown: a learned preconditioner whose output is not finite is
  rejected by the acceptance check and Jacobi-PCG finishes the solve (the
  result equals the plain solve's);
* non-finite elevations in valid cells: the fill gives the reference's
  result and the D8 engine the reference's error with (row, col)
  (flowinfo_cpu.cpp:1321-1328).
"""
import ctypes

import numpy as np
import pytest

from tests import surfaces

pytestmark = pytest.mark.gpu

ENOCONV, ETIMEOUT, EINVAL = 6, 7, 3


def _context_still_usable(port):
    import lsdtt_gb300 as G
    z = surfaces.fractal_pits(96)
    m = np.ones_like(z, np.uint8)
    got = G.fill_pits(z, m, 10.0, "oooo", 0.0).cpu().numpy()
    assert np.array_equal(got.view(np.uint32), port.fill_pits(z, m, 10.0, "oooo", 0.0).view(np.uint32))


def test_hillslope_iteration_cap_reports_nonconvergence(port):
    import lsdtt_gb300 as G
    z = port.noise_tilt_surface(128, 128, 30.0, 1, 0.0, 1.0, "nnon", 0.001)
    m = np.ones_like(z, np.uint8)
    with pytest.raises(G.GpuError) as ei:
        G.hillslope_linear_implicit(z, m, 30.0, "nnon", 0.5, 1000.0, max_iter=1)
    assert ei.value.status == ENOCONV and "did not reach" in str(ei.value)
    with pytest.raises(G.GpuError) as ei:
        G.hillslope_implicit(z, m, 30.0, "nnon", 0.5, 1.0, 1000.0, nonlinear=True, max_pcg_iter=1, max_outer=1)
    assert ei.value.status == ENOCONV
    model = G.LandscapeModel(z, m, 30.0, "nnon", timestep=1000.0, hillslope_diffusivity=0.5, hillslope_max_iter=1)
    with pytest.raises(G.GpuError) as ei:
        model.step()
    assert ei.value.status == ENOCONV
    model.close()
    _context_still_usable(port)


def test_ensemble_iteration_cap_reports_nonconvergence(port):
    import lsdtt_gb300 as G
    z = port.noise_tilt_surface(96, 112, 30.0, 2, 0.0, 1.0, "nnon", 0.001)
    ens = G.Ensemble([dict(z=z, cell_size=30.0, boundary_conditions="nnon", timestep=1000.0,
                           hillslope_diffusivity=0.5, hillslope_max_iter=1, fill_min_slope=1e-4)], use_graph=False)
    with pytest.raises(G.GpuError) as ei:
        ens.step()
    assert ei.value.status == ENOCONV and "did not reach" in str(ei.value)
    ens.close()
    _context_still_usable(port)


@pytest.mark.parametrize("entry,limit", [("lsdtt_gpu_selftest_grid_barrier", 1 << 14),
                                         ("lsdtt_gpu_selftest_mbarrier_wait", 1 << 12)])
def test_bounded_waits_give_up_and_report_timeout(port, entry, limit):
    import lsdtt_gb300 as G
    fn = getattr(G.lib(), entry)
    fn.argtypes = [ctypes.c_int32]
    fn.restype = ctypes.c_int
    status = fn(limit)
    assert status == ETIMEOUT, (entry, status, G.lib().lsdtt_gpu_last_error())
    assert fn(0) == EINVAL
    _context_still_usable(port)


def test_learned_solve_breakdown_falls_back_to_jacobi(port):
    """A network whose parameters are NaN makes the flexible PCG break down
    (r.z is not finite); the acceptance check rejects the iterate and
    Jacobi-PCG finishes every solve from zero: same surface as the plain
    solve."""
    import lsdtt_gb300 as G
    z = surfaces.fractal(128, 128, 20.0, 3)
    m = np.ones_like(z, np.uint8)
    net = G.UNet(128, 128, seed=1)
    net.set_params(np.full(net.n_params, np.nan, np.float32))
    plain, rep_p = G.hillslope_implicit(z, m, 5.0, "oooo", 0.01, 1.0, 2.5e4, nonlinear=True)
    got, rep = G.hillslope_implicit(z, m, 5.0, "oooo", 0.01, 1.0, 2.5e4, nonlinear=True, net=net)
    plain, got = plain.cpu().numpy(), got.cpu().numpy()
    rel = float(np.max(np.abs(got - plain) / np.maximum(np.abs(plain), 1.0)))
    print(f"breakdown: rejected {rep.rejected_solves}, fallback iterations {rep.fallback_iterations}, "
          f"network applications {rep.network_applications}, max rel vs plain {rel:.2e}, "
          f"bit-identical {np.array_equal(got.view(np.uint32), plain.view(np.uint32))}")
    assert rep.converged and rep.rejected_solves >= 1 and rep.fallback_iterations > 0
    assert rel < 1e-5
    net.close()
    _context_still_usable(port)


def test_nonfinite_elevation_in_a_valid_cell(port):
    """Infinite elevations are ordinary values to both fills (bit-exact at
    epsilon 0). A NaN elevation is kept as NaN by both; the reference's
    heap orders a NaN key arbitrarily, so around it the two fills may
    differ (counted, not bounded). The D8 engine rejects both with the
    reference's message and the cell's (row, col)."""
    import lsdtt_gb300 as G
    z = surfaces.fractal_pits(128)
    m = np.ones_like(z, np.uint8)
    z[70, 5] = np.inf
    z[40, 40] = -np.inf
    want = port.fill_pits(z, m, 10.0, "oooo", 0.0)
    got = G.fill_pits(z, m, 10.0, "oooo", 0.0).cpu().numpy()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    with pytest.raises(G.GpuError) as ei:
        G.FlowInfo(z, m, 10.0, "oooo", allow_pits_as_outlets=True)
    assert ei.value.status == EINVAL and "non-finite DEM value at row 40, col 40" in str(ei.value)
    zn = surfaces.fractal_pits(128)
    zn[20, 30] = np.nan
    for eps in (1e-4, 0.0):
        want = port.fill_pits(zn, m, 10.0, "oooo", eps)
        got = G.fill_pits(zn, m, 10.0, "oooo", eps).cpu().numpy()
        assert np.isnan(got[20, 30]) and np.isnan(want[20, 30])
        assert int(np.isnan(got).sum()) == 1
        same = got.view(np.uint32) == want.view(np.uint32)
        print(f"fill eps={eps} with a NaN cell: {int((~same).sum())} cells differ from the oracle")
    with pytest.raises(G.GpuError) as ei:
        G.FlowInfo(zn, m, 10.0, "oooo", allow_pits_as_outlets=True)
    assert ei.value.status == EINVAL and "non-finite DEM value at row 20, col 30" in str(ei.value)
    _context_still_usable(port)
