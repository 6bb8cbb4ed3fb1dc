"""The batched ensemble against its members run one at a time.

Every member of an lsdtt_gpu_ensemble must advance exactly as the
single-grid LandscapeModel advances it alone (which the LEM tests in
test_gpu_lem_path.py hold to the oracle). Members differ in shape (non-
square, not multiples of the tile or block size), boundary string
(including a periodic axis), fill on/off, stream-power exponent (n = 1, 1.5,
2), erodibility, diffusivity, uplift and hillslope on/off.

Bars: elevations within 1e-5 relative (the LEM bar; the only source of
difference is the order of the FP64 atomic reductions inside Jacobi-PCG);
the graph-replayed steps give the same result as eager steps to the same
bar; the schedule counters show the graph was captured and replayed.
"""
import numpy as np
import pytest

from tests import surfaces

pytestmark = pytest.mark.gpu

REL = 1e-5


def _members(port):
    specs = []
    z = port.noise_tilt_surface(96, 130, 30.0, 3, 0.0, 1.0, "nnon", 0.001)
    specs.append(dict(z=z, cell_size=30.0, boundary_conditions="nnon", timestep=1000.0, erodibility=1e-5,
                      m_exponent=0.5, n_exponent=1.0, uplift_rate=1e-3, hillslope_diffusivity=0.01,
                      fill_min_slope=1e-4))
    z = surfaces.fractal(200, 72, 40.0, 5).astype(np.float32)
    specs.append(dict(z=z, cell_size=10.0, boundary_conditions="oooo", timestep=500.0, erodibility=3e-5,
                      m_exponent=0.4, n_exponent=1.5, uplift_rate=2e-3, hillslope_diffusivity=0.05,
                      fill_min_slope=1e-4))
    z = port.noise_tilt_surface(128, 128, 20.0, 9, 0.0, 1.0, "nnon", 0.001)
    specs.append(dict(z=z, cell_size=20.0, boundary_conditions="nnon", timestep=1000.0, erodibility=1e-4,
                      m_exponent=0.6, n_exponent=2.0, uplift_rate=1e-4, hillslope_diffusivity=0.002,
                      fill_min_slope=0.0))
    z = surfaces.fractal(64, 80, 20.0, 11).astype(np.float32)
    specs.append(dict(z=z, cell_size=30.0, boundary_conditions="opop", timestep=1000.0, erodibility=2e-5,
                      m_exponent=0.45, n_exponent=1.0, uplift_rate=5e-4, hillslope_diffusivity=0.02,
                      fill_min_slope=1e-4))
    z = port.noise_tilt_surface(40, 48, 30.0, 13, 0.0, 1.0, "nnon", 0.001)
    specs.append(dict(z=z, cell_size=30.0, boundary_conditions="nnon", timestep=1000.0, erodibility=1e-5,
                      m_exponent=0.5, n_exponent=1.5, uplift_rate=1e-3, hillslope_diffusivity=0.01,
                      fill_min_slope=1e-4, enable_hillslope=False))
    return specs


def _alone(G, spec, steps):
    spec = dict(spec)
    z = spec.pop("z")
    cell = spec.pop("cell_size")
    bc = spec.pop("boundary_conditions")
    model = G.LandscapeModel(z, np.ones_like(z, np.uint8), cell, bc, **spec)
    its = []
    for _ in range(steps):
        its.append(model.step()["hillslope_iterations"])
    return model.z.cpu().numpy(), its


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(float(np.ptp(b)), 1.0))


@pytest.mark.parametrize("use_graph,sweep_mode", [(False, 0), (True, 0), (False, 1), (True, 1), (False, 2), (True, 2),
                                                     (False, 3), (True, 3)])
def test_ensemble_matches_members_alone(port, use_graph, sweep_mode):
    import lsdtt_gb300 as G
    specs = _members(port)
    steps = 6
    ens = G.Ensemble(specs, use_graph=use_graph)
    ens.override_schedule(sweep_mode=sweep_mode)
    for _ in range(steps - 1):
        ens.step()
    stats = ens.step(want_stats=True)
    info = ens.info()
    worst = 0.0
    for k, spec in enumerate(specs):
        z_alone, its = _alone(G, spec, steps)
        got = ens.get(k).cpu().numpy()
        err = _rel(got, z_alone)
        worst = max(worst, err)
        print(f"member {k} {spec['z'].shape} bc={spec['boundary_conditions']}: rel diff {err:.2e}; "
              f"PCG iterations alone {its[-1]} ensemble {stats[k]['hillslope_iterations']}")
        assert err <= REL, (k, err)
        # routing and stream power are the single-grid rules: report exactness
        if err == 0.0:
            print(f"member {k}: bit-identical")
        assert abs(stats[k]["hillslope_iterations"] - its[-1]) <= 4
    print("info", info)
    assert info["sweep_dataflow"] == sweep_mode
    if use_graph:
        assert info["graph_captures"] >= 1 and info["graph_replays"] >= steps - 2
    else:
        assert info["eager_steps"] == steps and info["graph_replays"] == 0


def test_graph_and_eager_agree_and_recover_from_overflow(port):
    import lsdtt_gb300 as G
    specs = _members(port)
    a = G.Ensemble(specs, use_graph=True)
    b = G.Ensemble(specs, use_graph=False)
    for _ in range(3):
        a.step()
        b.step()
    # Capture the next step with a schedule far too short for the fill and
    # the PCG: the replay after it must detect the overflow on the device,
    # undo the step and rerun it eagerly, then capture a fitting schedule.
    a.override_schedule(fill_pass_cap=4, hillslope_iteration_cap=4)
    before = a.info()
    for _ in range(5):
        a.step()
        b.step()
    after = a.info()
    print("info before", before, "after", after)
    assert after["graph_captures"] >= before["graph_captures"] + 2
    assert after["eager_steps"] >= before["eager_steps"] + 2
    for k in range(len(specs)):
        assert _rel(a.get(k).cpu().numpy(), b.get(k).cpu().numpy()) <= REL


def test_ensemble_errors():
    import lsdtt_gb300 as G
    z = np.zeros((16, 16), np.float32)
    with pytest.raises(G.GpuError):
        G.Ensemble([dict(z=z, cell_size=30.0, boundary_conditions="pppp")])
    with pytest.raises(G.GpuError):
        G.Ensemble([dict(z=z, cell_size=30.0, timestep=-1.0)])


def test_member_groups_give_the_same_result(port):
    """Captured steps with member groups (the deep members' sweep on a second
    stream beside the others' sweep and hillslope solve) against the same
    steps with one group: identical bits, and the grouped graph ran."""
    import lsdtt_gb300 as G
    specs = _members(port)
    z = port.noise_tilt_surface(384, 512, 30.0, 17, 0.0, 1.0, "nnon", 0.001)
    specs.append(dict(z=z, cell_size=30.0, boundary_conditions="nnon", timestep=1000.0, erodibility=2e-5,
                      m_exponent=0.5, n_exponent=1.5, uplift_rate=1e-3, hillslope_diffusivity=0.01,
                      fill_min_slope=1e-4))
    out = {}
    for groups in (True, False):
        ens = G.Ensemble(specs, use_graph=True)
        ens.override_schedule(sweep_mode=3)
        ens.set_member_groups(groups)
        ens.step(4)
        info = ens.info()
        assert info["graph_replays"] >= 3
        if groups:
            assert info["deep_members"] > 0, info
        else:
            assert info["deep_members"] == 0
        out[groups] = [ens.get(k).cpu().numpy() for k in range(len(specs))]
        ens.close()
    for k, (a, b) in enumerate(zip(out[True], out[False])):
        assert np.array_equal(a, b), f"member {k}: max |diff| {np.max(np.abs(a - b))}"


def test_steps_are_deterministic(port):
    """Two fresh ensembles stepped eagerly give identical bits: the fill
    relaxes its active tiles colour by colour (no two tiles of a colour are
    neighbours), so no result depends on which tiles ran first."""
    import lsdtt_gb300 as G
    specs = _members(port)
    # enough tiles for a pass to run in several waves
    z = port.noise_tilt_surface(384, 512, 30.0, 17, 0.0, 1.0, "nnon", 0.001)
    specs.append(dict(z=z, cell_size=30.0, boundary_conditions="nnon", timestep=1000.0, erodibility=2e-5,
                      m_exponent=0.5, n_exponent=1.5, uplift_rate=1e-3, hillslope_diffusivity=0.01,
                      fill_min_slope=1e-4))
    runs = []
    for _ in range(2):
        ens = G.Ensemble(specs, use_graph=False)
        ens.step(2)
        runs.append([ens.get(k).cpu().numpy() for k in range(len(specs))])
        ens.close()
    for k, (a, b) in enumerate(zip(*runs)):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), f"member {k}"
