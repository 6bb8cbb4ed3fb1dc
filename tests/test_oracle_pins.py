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
