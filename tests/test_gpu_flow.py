"""GPU D8 engine parity: receivers, directions, donor counts, outlets,
topological order, s-vector, contributing counts and accumulation, bit for
bit, against (a) the reference's golden FNV-1a pins on its 17 fixtures and
(b) the CPU oracle on seeded larger surfaces."""
import json
import os

import numpy as np
import pytest

from tests.golden import d8_fixtures as F
from tests import surfaces

pytestmark = pytest.mark.gpu

PINS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "d8_identity_pins.json")))["pins"]


def gpu_result(fx, cfg):
    import lsdtt_gb300 as G
    _, topo, sv, acyc = cfg
    fi = G.FlowInfo(fx["z"], fx["mask"], fx["cell"], fx["bc"],
                    interior_nodata_is_outlet=fx["interior_nodata_is_outlet"], require_acyclic_graph=acyc,
                    build_topological_order=topo, build_s_vector=sv,
                    allow_pits_as_outlets=fx["pits_as_outlets"], forced_outlet_flats=list(fx["forced"]))
    res = dict(receiver=fi.receiver().cpu().numpy(), direction=fi.direction().cpu().numpy(),
               donors=fi.donor_count().cpu().numpy(), outlets=fi.outlets().cpu().numpy(),
               has_topo=fi.has_topological_order(), has_sv=fi.has_s_vector())
    if res["has_topo"]:
        res["topo"] = fi.topological_order().cpu().numpy()
        res["accum_area"] = fi.accumulate().cpu().numpy()
        res["accum_w"] = fi.accumulate(F.test_weights(fx["z"].size)).cpu().numpy()
    if res["has_sv"]:
        res["s_vector"] = fi.s_vector().cpu().numpy()
        res["sv_start"] = fi.s_vector_start().cpu().numpy()
        res["sv_size"] = fi.s_vector_size().cpu().numpy().astype(np.uint64)
    fi.close()
    return res


@pytest.mark.parametrize("spec", F.SPECS, ids=[s[0] for s in F.SPECS])
def test_gpu_matches_reference_pins(spec):
    fx = F.make_fixture(spec)
    for cfg in F.CONFIGS:
        key = f"{fx['name']}/{cfg[0]}"
        got = F.hash_components(fx, gpu_result(fx, cfg))
        want = {k: int(v, 16) for k, v in PINS[key].items()}
        bad = {k: (hex(got[k]), hex(want[k])) for k in want if got[k] != want[k]}
        assert not bad, f"{key}: {bad}"


def _compare_with_oracle(port, z, mask, cell, bc, pits=True):
    import lsdtt_gb300 as G
    want = port.flowinfo(z, mask, cell, bc, allow_pits_as_outlets=pits)
    fi = G.FlowInfo(z, mask, cell, bc, allow_pits_as_outlets=pits)
    n_mismatch = {}
    for name, got in (("receiver", fi.receiver()), ("direction", fi.direction()), ("donors", fi.donor_count()),
                      ("outlets", fi.outlets()), ("topo", fi.topological_order()), ("s_vector", fi.s_vector()),
                      ("sv_start", fi.s_vector_start()), ("accum", fi.accumulate())):
        g = got.cpu().numpy()
        w = want[name]
        assert g.shape == w.shape, name
        n_mismatch[name] = int(np.count_nonzero(g.view(np.uint8).reshape(g.size, -1) !=
                                                w.astype(g.dtype).view(np.uint8).reshape(w.size, -1)))
    g = fi.s_vector_size().cpu().numpy().astype(np.uint64)
    n_mismatch["sv_size"] = int(np.count_nonzero(g != want["sv_size"]))
    fi.close()
    assert all(v == 0 for v in n_mismatch.values()), n_mismatch


def test_gpu_noise_tilt_512(port):
    z = port.noise_tilt_surface(512, 512, 30.0, 1, 0.0, 1.0, "nnon", 0.001)
    m = np.ones_like(z, np.uint8)
    f = port.fill_pits(z, m, 30.0, "nnon", 1e-4)
    _compare_with_oracle(port, f, m, 30.0, "nnon")
    _compare_with_oracle(port, z, m, 30.0, "nnon")  # unfilled: pits become outlets


def test_gpu_fractal_pits_1024(port):
    z = surfaces.fractal_pits(1024)
    m = np.ones_like(z, np.uint8)
    f = port.fill_pits(z, m, 10.0, "oooo", 1e-4)
    _compare_with_oracle(port, f, m, 10.0, "oooo")


def test_gpu_fractal_holes_periodic(port):
    rng = np.random.default_rng(3)
    z = surfaces.fractal(300, 420, 300.0, 5)
    m = (rng.random(z.shape) > 0.03).astype(np.uint8)
    z[m == 0] = -9999.0
    for bc in ("popo", "nnnn", "onbn"):
        _compare_with_oracle(port, z, m, 5.0, bc)


def test_gpu_unresolved_sink_message():
    import lsdtt_gb300 as G
    z = np.full((5, 6), 10.0, np.float32)
    z[2, 3] = 1.0
    m = np.ones_like(z, np.uint8)
    with pytest.raises(G.GpuError) as e:
        G.FlowInfo(z, m, 10.0, "nnnn")
    assert "could not assign a receiver at row 0, col 0" in str(e.value)
    assert e.value.status == G.EUNRESOLVED


def _adversarial_surfaces():
    """Elevations aimed at every branch of the receiver ranking."""
    rng = np.random.default_rng(17)
    shape = (97, 101)  # crosses 32-cell tile seams, ragged last tile
    r, c = np.mgrid[0:shape[0], 0:shape[1]].astype(np.float64)
    out = {}
    # exact ties inside a class and between classes
    out["small_ints"] = rng.integers(0, 4, shape).astype(np.float32)
    # planes whose best cardinal and diagonal drops are consecutive convergents
    # of sqrt2 (8119/5741, 19601/13860): cross-class near-ties below 2^-18
    p1 = 2.0e6 + 5741.0 * (shape[0] - r) + 2378.0 * (shape[1] - c)
    p2 = 8.0e6 + 13860.0 * (shape[0] - r) + 5741.0 * (shape[1] - c)
    out["sqrt2_planes"] = np.where(r < shape[0] // 2, p1, p2).astype(np.float32)
    # drops that dwarf tiny, zero, subnormal and signed-zero neighbours
    pool = np.array([1e9, 3e8, 1.0, 0.0, -0.0, 1e-30, -1e-30, 2e-38, 1e-44, -1e-44, 5e-7, -3.0], np.float32)
    out["magnitudes"] = pool[rng.integers(0, pool.size, shape)]
    # fractal relief with infinities and NaNs under masked cells (a valid
    # cell must hold a finite value)
    f = surfaces.fractal(shape[0], shape[1], 300.0, 7).astype(np.float32) - 150.0
    pick = rng.random(shape)
    f[pick < 0.004] = np.inf
    f[(pick >= 0.004) & (pick < 0.008)] = -np.inf
    f[(pick >= 0.008) & (pick < 0.010)] = np.nan
    out["nonfinite"] = f
    return out


@pytest.mark.parametrize("name", ["small_ints", "sqrt2_planes", "magnitudes", "nonfinite"])
def test_gpu_receivers_adversarial(port, name):
    z = _adversarial_surfaces()[name]
    rng = np.random.default_rng(5)
    full = np.ones_like(z, np.uint8)
    holes = (rng.random(z.shape) > 0.05).astype(np.uint8)
    for m in (full, holes):
        m = m & np.isfinite(z).astype(np.uint8)
        for cell, bc in ((10.0, "oooo"), (3.0, "popo"), (0.7, "nnon")):
            _compare_with_oracle(port, z, m, cell, bc)
