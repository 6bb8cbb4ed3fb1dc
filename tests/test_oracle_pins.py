"""The CPU oracle against the reference's golden FNV-1a pins
(tests/cpp/test_flow_d8_identity.cpp k_pins, extracted to
tests/golden/d8_identity_pins.json): 17 fixtures x 4 option configurations x
8 components (receiver, direction, donors, outlets, topo, svector, area,
weighted)."""
import json
import os

import numpy as np
import pytest

from tests.golden import d8_fixtures as F

PINS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "d8_identity_pins.json")))["pins"]


def oracle_result(port, fx, cfg, n_threads=1):
    _, topo, sv, acyc = cfg
    kw = dict(bc=fx["bc"], interior_nodata_is_outlet=fx["interior_nodata_is_outlet"],
              allow_pits_as_outlets=fx["pits_as_outlets"], build_topo=topo, build_sv=sv,
              require_acyclic=acyc, forced=fx["forced"], n_threads=n_threads)
    res = port.flowinfo(fx["z"], fx["mask"], fx["cell"], **kw)
    if res["has_topo"]:
        res["accum_area"] = res["accum"]
        res["accum_w"] = port.flowinfo(fx["z"], fx["mask"], fx["cell"], weights=F.test_weights(fx["z"].size),
                                       **kw)["accum"]
    return res


@pytest.mark.parametrize("spec", F.SPECS, ids=[s[0] for s in F.SPECS])
def test_oracle_matches_reference_pins(port, spec):
    fx = F.make_fixture(spec)
    for cfg in F.CONFIGS:
        key = f"{fx['name']}/{cfg[0]}"
        got = F.hash_components(fx, oracle_result(port, fx, cfg))
        want = {k: int(v, 16) for k, v in PINS[key].items()}
        bad = {k: (hex(got[k]), hex(want[k])) for k in want if got[k] != want[k]}
        assert not bad, f"{key}: {bad}"


@pytest.mark.parametrize("spec", F.SPECS[:4], ids=[s[0] for s in F.SPECS[:4]])
def test_oracle_thread_count_invariance(port, spec):
    fx = F.make_fixture(spec)
    a = oracle_result(port, fx, F.CONFIGS[0], n_threads=1)
    b = oracle_result(port, fx, F.CONFIGS[0], n_threads=3)
    for k in ("receiver", "direction", "topo", "s_vector"):
        assert np.array_equal(a[k], b[k])


@pytest.mark.parametrize("shape", [(128, 128), (96, 160)])
def test_routing_properties_hold_for_the_oracle(port, shape):
    """The size-independent routing properties that the GPU test checks at
    8192 x 8192 hold for the oracle's outputs (fractal with pits, 10 m)."""
    from tests import routing_props as RP
    from tests import surfaces
    nr, nc = shape
    z = surfaces.add_pits(surfaces.fractal(nr, nc, 1000.0, 7), 40, 7)
    m = np.ones_like(z, np.uint8)
    filled = port.fill_pits(z, m, 10.0, "oooo", 1e-4)
    RP.check_fill(z, filled)
    w = port.flowinfo(filled, m, 10.0, "oooo", allow_pits_as_outlets=True)
    RP.check_flow(filled, 10.0, w["receiver"], w["direction"], w["donors"], w["outlets"], w["topo"],
                  w["s_vector"], w["sv_start"], w["sv_size"], w["accum"])


def test_routing_properties_catch_planted_mistakes(port):
    """Each planted mistake in the oracle's outputs trips a property."""
    from tests import routing_props as RP
    from tests import surfaces
    z = surfaces.add_pits(surfaces.fractal(64, 64, 1000.0, 3), 10, 3)
    m = np.ones_like(z, np.uint8)
    filled = port.fill_pits(z, m, 10.0, "oooo", 1e-4)
    w = port.flowinfo(filled, m, 10.0, "oooo", allow_pits_as_outlets=True)
    args = ["receiver", "direction", "donors", "outlets", "topo", "s_vector", "sv_start", "sv_size", "accum"]

    def flow(**bad):
        v = {k: bad.get(k, w[k]) for k in args}
        RP.check_flow(filled, 10.0, *[v[k] for k in args])

    flow()  # unmodified: passes
    c = int(np.flatnonzero(w["receiver"] >= 0)[0])
    r = int(w["receiver"][c])
    pit = filled.copy()
    pit[32, 32] = z[32, 32] - 10.0
    with pytest.raises(AssertionError):
        RP.check_fill(z, pit)
    topo = w["topo"].copy()
    i, j = np.flatnonzero(topo == c)[0], np.flatnonzero(topo == r)[0]
    topo[i], topo[j] = topo[j], topo[i]
    sz = w["sv_size"].copy()
    sz[c] += 1
    acc = w["accum"].copy()
    acc[c] = np.nextafter(acc[c], np.inf)
    d = w["direction"].copy()
    d[c] = (d[c] + 1) % 8
    for bad in (dict(topo=topo), dict(sv_size=sz), dict(accum=acc), dict(direction=d)):
        with pytest.raises(AssertionError):
            flow(**bad)
