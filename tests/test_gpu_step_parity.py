"""The benchmarked LEM step against the composed oracle, stage by stage.

The composed oracle for one step is the reference's per-step chain
(fill_pits -> run_lem_step: lsdtt_flowinfo, compute_d8_stream_power_incision,
the implicit linear hillslope, uplift and boundary restore;
lem_cpu.cpp:285-732), with the hillslope solved in FP64 (the restatement
in oracle/hillslope.py; the reference's Eigen build is not available).

Each stage is pinned on the same input:

* the fill: GPU fill of the oracle's step input bit for bit at every step
  against the oracle's priority flood with heap ties taken in (row, col)
  order -- the GPU's rule. The reference's binary heap orders entries of
  equal value by its internal layout (on these LEM inputs thousands of
  equal-value pops per step, about half of them first-in-first-out), which
  no parallel fill can reproduce; the cells where such a tie decided a
  discovery (7 of 452,251 raised cells over config 1's 200 steps) are
  counted against the reference's own order;
* everything after the fill (routing, stream power, hillslope, uplift,
  restore, statistics): the GPU step with its fill switched off, fed the
  oracle's filled surface, against the oracle's rest of the step, within
  1e-5 relative (REL_TOL) at every step;
* the ensemble (the benchmark's own code path, CUDA-graph replays included)
  the same way on members drawn by the benchmark's own generator, plus its
  fill (also replayed from its graph) against the single-grid fill and the
  oracle's, bit for bit.

A free-running GPU trajectory (fill included) is reported beside it: the
FP32 hillslope solve differs from the FP64 one in the last bits, and where
such a difference moves a cell across a fill decision the trajectories part.
"""
import numpy as np
import pytest

import oracle
import oracle.hillslope as H

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5        # elevations, relative (max(|z|, 1)), as the reference's contract states


def _rel(got, want):
    return float(np.max(np.abs(got.astype(np.float64) - want) / np.maximum(np.abs(want), 1.0)))


def oracle_rest(port, f, m, cell, bc, K, mexp, nexp, dt, U, D, bf):
    """The step after the fill: stream power on the filled surface, the
    implicit linear hillslope (FP64 CG to a 1e-12 relative residual, a
    converged solve), uplift, boundary restore, statistics."""
    zsp = port.stream_power(f, m, cell, bc, K, mexp, nexp, dt)
    zh, _, _ = H.linear_step(zsp, m, cell, bc, D, dt, solver="pcg", rel_tol=1e-12)
    return oracle.lem_finish(zh, f, m, U, dt, bf)


def fill_vs(got, want):
    return int((got.view(np.uint32) != want.view(np.uint32)).sum())


def fill_mismatch(got, want, z):
    raised = want != z
    diff = got.view(np.uint32) != want.view(np.uint32)
    return int(diff.sum()), int(raised.sum()), int((raised != (got != z)).sum())


def test_config1_200_steps_stagewise(port):
    """Config 1 as specified: 512 x 512 noise + tilt (the reference's
    generator), dx 30 m, bc nnon, K 1e-5, m 0.5, n 1, U 1e-3, D 0.01,
    dt 1000 yr, epsilon fill 1e-4 every step, 200 steps."""
    import torch
    import lsdtt_gb300 as G
    cell, bc, K, mexp, nexp, dt, U, D = 30.0, "nnon", 1e-5, 0.5, 1.0, 1000.0, 1e-3, 0.01
    z = port.noise_tilt_surface(512, 512, cell, 1, 0.0, 1.0, bc, 0.001)
    m = np.ones_like(z, np.uint8)
    bf = port.boundary_flats(m, bc)
    rest = G.LandscapeModel(z, m, cell, bc, timestep=dt, erodibility=K, m_exponent=mexp, n_exponent=nexp,
                            uplift_rate=U, hillslope_diffusivity=D, fill_min_slope=0.0)
    free = G.LandscapeModel(z, m, cell, bc, timestep=dt, erodibility=K, m_exponent=mexp, n_exponent=nexp,
                            uplift_rate=U, hillslope_diffusivity=D, fill_min_slope=1e-4)
    worst_rest, worst_cells, worst_status, sum_diff, sum_raised, tie_rule_diff = 0.0, 0.0, 0, 0, 0, 0
    for step in range(200):
        f = port.fill_pits(z, m, cell, bc, 1e-4)
        gf = G.fill_pits(z, m, cell, bc, 1e-4).cpu().numpy()
        tie_rule_diff += fill_vs(gf, port.fill_pits_index_ties(z, m, cell, bc, 1e-4))
        nd, nraised, nstatus = fill_mismatch(gf, f, z)
        sum_diff += nd
        sum_raised += nraised
        worst_cells = max(worst_cells, nd / z.size)
        worst_status = max(worst_status, nstatus)
        rest.z.copy_(torch.from_numpy(f).cuda())
        st = rest.step()
        z, ost = oracle_rest(port, f, m, cell, bc, K, mexp, nexp, dt, U, D, bf)
        err = _rel(rest.z.cpu().numpy(), z)
        worst_rest = max(worst_rest, err)
        assert err < REL_TOL, (step, err)
        assert abs(st["max_local_elevation_change"] - ost[2]) <= 1e-5 * max(1.0, abs(float(ost[2]))), step
        free.step()
    got = free.z.cpu().numpy()
    relief = float(np.ptp(z))
    drift = float(np.max(np.abs(got - z))) / relief
    mean_drift = abs(float(got.mean()) - float(z.mean())) / relief
    print(f"config 1, 200 steps: after-fill stages max rel {worst_rest:.2e}; fill: {tie_rule_diff} cells differ "
          f"from the oracle with (row, col) heap ties over the run; {sum_diff} of {sum_raised} raised cells differ "
          f"from the reference's heap order (heap ties), raised/unraised status in at most {worst_status} cells; "
          f"free-running GPU vs oracle after 200 steps: max |dz| {drift:.2e} of the relief, mean {mean_drift:.2e}")
    assert tie_rule_diff == 0
    assert sum_diff <= 1e-4 * sum_raised
    assert mean_drift < 1e-4
    rest.close()
    free.close()


def _bench_members():
    """Four members of the benchmark's own ensemble (bench.ensemble_specs):
    the first with n = 1, 1.5 and 2 among the smaller members, and the
    largest member."""
    import bench
    specs = bench.ensemble_specs(256)
    largest = max(range(len(specs)), key=lambda i: specs[i]["z"].size)
    picked = [largest]
    for n in (1.0, 1.5, 2.0):
        for i, s in enumerate(specs):
            if s["n_exponent"] == n and i not in picked and s["z"].size <= 400 * 400:
                picked.append(i)
                break
    return [specs[i] for i in picked]


def test_bench_ensemble_members_stagewise(port):
    """Members of the benchmark ensemble stepped 20 times inside one
    lsdtt_gpu_ensemble (the first step eager, the rest CUDA-graph replays),
    each step fed the oracle's filled surface, against the oracle's rest of
    the step; and the ensemble's own fill (a member whose erosion,
    hillslope and uplift are off steps to its filled surface) against the
    single-grid GPU fill (bit for bit) and the oracle's fill (bit for bit
    with (row, col) heap ties; the fill ensemble also replays its CUDA
    graph)."""
    import lsdtt_gb300 as G
    members = _bench_members()
    ens = G.Ensemble([dict(s, fill_min_slope=0.0) for s in members], use_graph=True)
    fills = G.Ensemble([dict(s, fill_min_slope=1e-4, erodibility=0.0, enable_hillslope=False, uplift_rate=0.0)
                        for s in members], use_graph=True)
    zs = [s["z"].copy() for s in members]
    masks = [np.ones_like(z, np.uint8) for z in zs]
    bfs = [port.boundary_flats(m, s["boundary_conditions"]) for s, m in zip(members, masks)]
    worst_rest, worst_cells, sum_diff, sum_raised, tie_rule_diff = 0.0, 0.0, 0, 0, 0
    for step in range(20):
        filled = []
        for k, s in enumerate(members):
            f = port.fill_pits(zs[k], masks[k], s["cell_size"], s["boundary_conditions"], 1e-4)
            filled.append(f)
            ens.set(k, f)
            fills.set(k, zs[k])
        ens.step()
        fills.step()
        for k, s in enumerate(members):
            ef = fills.get(k).cpu().numpy()
            gf = G.fill_pits(zs[k], masks[k], s["cell_size"], s["boundary_conditions"], 1e-4).cpu().numpy()
            assert np.array_equal(ef.view(np.uint32), gf.view(np.uint32)), (step, k)
            tie_rule_diff += fill_vs(ef, port.fill_pits_index_ties(zs[k], masks[k], s["cell_size"],
                                                                   s["boundary_conditions"], 1e-4))
            nd, nraised, _ = fill_mismatch(ef, filled[k], zs[k])
            sum_diff += nd
            sum_raised += nraised
            worst_cells = max(worst_cells, nd / zs[k].size)
            zs[k], _ = oracle_rest(port, filled[k], masks[k], s["cell_size"], s["boundary_conditions"],
                                   s["erodibility"], s["m_exponent"], s["n_exponent"], s["timestep"],
                                   s["uplift_rate"], s["hillslope_diffusivity"], bfs[k])
            err = _rel(ens.get(k).cpu().numpy(), zs[k])
            worst_rest = max(worst_rest, err)
            assert err < REL_TOL, (step, k, members[k]["z"].shape, members[k]["n_exponent"], err)
    info = ens.info()
    print(f"bench members {[(s['z'].shape, s['n_exponent']) for s in members]}: after-fill stages max rel "
          f"{worst_rest:.2e} over 20 steps ({info['graph_replays']} graph replays); ensemble fill == single-grid "
          f"fill; {tie_rule_diff} cells differ from the oracle with (row, col) heap ties, {sum_diff} of "
          f"{sum_raised} raised cells from the reference's heap order")
    assert info["graph_replays"] >= 18
    assert fills.info()["graph_replays"] >= 18
    assert tie_rule_diff == 0
    assert sum_diff <= 1e-4 * sum_raised
    ens.close()
    fills.close()


def test_roering_512_against_fp64_newton():
    """One Roering (nonlinear) implicit hillslope step at 512 x 512 (four
    x sixteen 128 x 32 operator tiles, steep enough faces for the line
    search) against the stored FP64 Newton + sparse LU restatement
    (tests/golden/make_roering_fixture.py)."""
    import os
    import lsdtt_gb300 as G
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "roering_512.npz"))
    z, want = d["z"], d["out"]
    m = np.ones_like(z, np.uint8)
    got, rep = G.hillslope_implicit(z, m, float(d["cell"]), str(d["bc"]), float(d["D"]), float(d["Sc"]),
                                    float(d["dt"]), nonlinear=True)
    err = _rel(got.cpu().numpy(), want)
    print(f"Roering 512^2: max rel {err:.2e}, PCG iterations {rep.iterations}; oracle sub-steps {int(d['n_sub'])}")
    assert rep.converged
    assert err < REL_TOL
