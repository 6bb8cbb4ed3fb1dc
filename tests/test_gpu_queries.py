"""The lsdtt_flow_base query rasters on the GPU engine (lsdtt_gpu_flow_query)
against the oracle's restatement of lsdtt_flowinfo's own
(src/cpu/lsdtt_flowinfo_cpu.cpp:2255-2965; the restatement is held bit-equal
to the compiled reference in tests/test_oracle_vs_reference.py): data, mask
and the donor raster, bit for bit, on surfaces with pits, interior holes and
a periodic axis."""
import numpy as np
import pytest

from tests import surfaces

pytestmark = pytest.mark.gpu

KINDS = ["distance_from_outlet", "height_above_channel", "height_above_channel_mask", "distance_to_channel",
         "height_to_farthest_ridge", "distance_to_farthest_ridge", "downstream_path_sum", "upslope_sum",
         "upslope_mean"]


def _cases(port):
    z1 = port.noise_tilt_surface(160, 224, 30.0, 4, 0.0, 1.0, "nnon", 0.001)
    z2 = surfaces.fractal_pits(192, seed=5)
    m2 = np.ones_like(z2, np.uint8)
    m2[50:60, 70:95] = 0
    z3 = surfaces.add_pits(surfaces.fractal(144, 176, 150.0, 6), 30, 6)
    one = lambda z: np.ones_like(z, np.uint8)  # noqa: E731
    return [("noise_tilt_nnon", z1, one(z1), 30.0, "nnon"), ("fractal_holes_oooo", z2, m2, 10.0, "oooo"),
            ("fractal_popo", z3, one(z3), 10.0, "popo")]


@pytest.mark.parametrize("kind", KINDS)
def test_query_raster_matches_oracle(port, kind):
    import lsdtt_gb300 as G
    for name, z, m, cell, bc in _cases(port):
        f = port.fill_pits(z, m, cell, bc, 1e-4)
        rng = np.random.default_rng(len(name))
        vals = rng.uniform(-5.0, 50.0, z.shape).astype(np.float32)
        vm = (rng.uniform(0, 1, z.shape) > 0.05).astype(np.uint8)
        cm = (rng.uniform(0, 1, z.shape) > 0.97).astype(np.uint8)
        want = port.flow_query(kind, f, m, cell, bc, values=vals, vmask=vm, cmask=cm, threshold=25,
                               include_self=(len(name) % 2 == 0))
        fi = G.FlowInfo(f, m, cell, bc, allow_pits_as_outlets=True)
        got, gm, gd = fi.query(kind, values=vals, value_mask=vm, channel_mask=cm, threshold=25,
                               include_self=(len(name) % 2 == 0))
        got, gm = got.cpu().numpy(), gm.cpu().numpy()
        fi.close()
        assert np.array_equal(gm, want[1]), (name, kind, int((gm != want[1]).sum()))
        diff = got.view(np.uint32) != want[0].view(np.uint32)
        assert not diff.any(), (name, kind, int(diff.sum()), float(np.max(np.abs(got - want[0]))))
        if want[2] is not None:
            assert np.array_equal(gd.cpu().numpy().ravel(), want[2]), (name, kind)
