"""The restated oracle (oracle/lsdtt_oracle.cpp) against the reference's own
sources compiled where they lie (oracle/_ref/liblsdtt_ref.so, built by
`make -C oracle ref` from an lsdtt3 checkout): bit for bit on every output of
the path it restates.

* fill_pits at epsilon 1e-4 and 0, on the LEM's noise + tilt surface ("nnon"),
  a fractal with pits ("oooo"), a periodic fractal ("popo" and "opop") and a
  grid with interior nodata -- raster_flow_preprocessing_cpu.cpp:416-589,
  707-782, 1203;
* lsdtt_flowinfo: receivers, directions, donor counts, outlets, Kahn order,
  s-vector, starts, sizes and accumulated area -- flowinfo_cpu.cpp:197-253,
  1077-1731, 1979-2046;
* compute_d8_stream_power_incision at n = 1, 1.5, 2 --
  stream_power_cpu.cpp:159-326.

Skipped where the reference library is absent (the GPU machine has no
checkout). The GPU parity tests check the GPU against the restatement; this
file is what ties the restatement to the reference itself."""
import numpy as np
import pytest

import oracle
from tests import surfaces

pytestmark = pytest.mark.skipif(not oracle.ref_available(), reason="oracle/_ref not built (no lsdtt3 checkout)")


def _bits_equal(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    if a.dtype.kind == "f":
        return a.shape == b.shape and np.array_equal(a.view(np.uint32 if a.itemsize == 4 else np.uint64),
                                                     b.view(np.uint32 if b.itemsize == 4 else np.uint64))
    return np.array_equal(a, b)


def _surfaces(port):
    z1 = port.noise_tilt_surface(256, 256, 30.0, 1, 0.0, 1.0, "nnon", 0.001)
    fr = surfaces.fractal_pits(256)
    per = surfaces.add_pits(surfaces.fractal(160, 224, 300.0, 5), 60, 5)
    holes = surfaces.fractal_pits(192, seed=9)
    mh = np.ones_like(holes, np.uint8)
    mh[40:52, 60:90] = 0
    mh[120, 10:30] = 0
    one = lambda z: np.ones_like(z, np.uint8)  # noqa: E731
    return [("noise_tilt_nnon", z1, one(z1), 30.0, "nnon"),
            ("fractal_pits_oooo", fr, one(fr), 10.0, "oooo"),
            ("fractal_popo", per, one(per), 10.0, "popo"),
            ("fractal_opop", per, one(per), 10.0, "opop"),
            ("fractal_holes_oooo", holes, mh, 10.0, "oooo")]


@pytest.fixture(scope="module")
def ref():
    return oracle.ref()


@pytest.mark.parametrize("eps", [1e-4, 0.0])
def test_fill_port_equals_reference(port, ref, eps):
    for name, z, m, cell, bc in _surfaces(port):
        a = port.fill_pits(z, m, cell, bc, eps)
        b = ref.fill_pits(z, m, cell, bc, eps)
        assert _bits_equal(a, b), (name, eps, int(np.count_nonzero(a != b)))


def test_flowinfo_port_equals_reference(port, ref):
    for name, z, m, cell, bc in _surfaces(port):
        f = port.fill_pits(z, m, cell, bc, 1e-4)
        a = port.flowinfo(f, m, cell, bc, allow_pits_as_outlets=True)
        b = ref.flowinfo(f, m, cell, bc, allow_pits_as_outlets=True)
        for key in ("receiver", "direction", "donors", "outlets", "topo", "s_vector", "sv_start", "sv_size",
                    "accum"):
            assert _bits_equal(a[key], b[key]), (name, key)


@pytest.mark.parametrize("n_exp", [1.0, 1.5, 2.0])
def test_stream_power_port_equals_reference(port, ref, n_exp):
    for name, z, m, cell, bc in _surfaces(port)[:3]:
        f = port.fill_pits(z, m, cell, bc, 1e-4)
        a = port.stream_power(f, m, cell, bc, 2e-5, 0.45, n_exp, 500.0)
        b = ref.stream_power(f, m, cell, bc, 2e-5, 0.45, n_exp, 500.0)
        assert _bits_equal(a, b), (name, n_exp)


def test_fluvial_lem_steps_port_equal_reference(port, ref):
    """Five fluvial LEM steps with the per-step epsilon fill: the port's
    composition (fill -> stream power -> uplift / boundary restore /
    statistics) against the reference's own run_lem_step with hillslopes
    off (lem_cpu.cpp:285-732), each fed its own previous output."""
    z0 = port.noise_tilt_surface(128, 160, 30.0, 3, 0.0, 1.0, "nnon", 0.001)
    m = np.ones_like(z0, np.uint8)
    bf = port.boundary_flats(m, "nnon")
    assert np.array_equal(bf, ref.boundary_flats(m, "nnon"))
    za, zb = z0.copy(), z0.copy()
    for _ in range(5):
        fa = port.fill_pits(za, m, 30.0, "nnon", 1e-4)
        za, sa = oracle.lem_finish(port.stream_power(fa, m, 30.0, "nnon", 1e-5, 0.5, 1.0, 1000.0), fa, m, 1e-3,
                                   1000.0, bf)
        zb, sb = ref.lem_step_fluvial(ref.fill_pits(zb, m, 30.0, "nnon", 1e-4), m, 30.0, "nnon", 1000.0, 1e-5,
                                      0.5, 1.0, 1e-3, bf)
        assert _bits_equal(za, zb)
        assert _bits_equal(sa, sb)


def test_flow_queries_port_equal_reference(port, ref):
    """The lsdtt_flow_base query rasters (flowinfo_cpu.cpp:2255-2965): data,
    mask and the donor raster, every kind, on every surface."""
    for name, z, m, cell, bc in _surfaces(port):
        f = port.fill_pits(z, m, cell, bc, 1e-4)
        rng = np.random.default_rng(len(name))
        vals = rng.uniform(-5.0, 50.0, z.shape).astype(np.float32)
        vm = (rng.uniform(0, 1, z.shape) > 0.05).astype(np.uint8)
        cm = (rng.uniform(0, 1, z.shape) > 0.97).astype(np.uint8)
        for kind in port.QUERY_KINDS:
            a = port.flow_query(kind, f, m, cell, bc, values=vals, vmask=vm, cmask=cm, threshold=25)
            b = ref.flow_query(kind, f, m, cell, bc, values=vals, vmask=vm, cmask=cm, threshold=25)
            assert _bits_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), (name, kind)
            if a[2] is not None:
                assert np.array_equal(a[2], b[2]), (name, kind)


def test_dinf_port_equals_reference(port, ref):
    """The D-infinity lsdtt_flowgraph_cpu (receivers, weights, facet slopes
    and bearings, donor counts, topological order), its accumulate and
    compute_dinf_stream_power_incision at n = 1, 1.5, 2."""
    for name, z, m, cell, bc in _surfaces(port)[:4]:
        f = port.fill_pits(z, m, cell, bc, 1e-4)
        a = port.dinf_graph(f, m, cell, bc)
        b = ref.dinf_graph(f, m, cell, bc)
        for key in a:
            assert _bits_equal(a[key], b[key]), (name, key)
        assert _bits_equal(port.dinf_accumulate(f, m, cell, bc), ref.dinf_accumulate(f, m, cell, bc)), name
        for n_exp in (1.0, 1.5, 2.0):
            assert _bits_equal(port.dinf_stream_power(f, m, cell, bc, 2e-5, 0.45, n_exp, 500.0),
                               ref.dinf_stream_power(f, m, cell, bc, 2e-5, 0.45, n_exp, 500.0)), (name, n_exp)


def test_index_tie_variant_only_changes_ties(port):
    """The oracle's (row, col) heap-tie variant (the GPU fill's rule) equals
    the restatement of the reference wherever no two heap entries of equal
    value compete: on surfaces with continuous random elevations."""
    from tests import surfaces
    one = lambda z: np.ones_like(z, np.uint8)  # noqa: E731
    for z, cell, bc in [(port.noise_tilt_surface(256, 256, 30.0, 1, 0.0, 1.0, "nnon", 0.001), 30.0, "nnon"),
                        (surfaces.fractal_pits(256), 10.0, "oooo"),
                        (surfaces.add_pits(surfaces.fractal(96, 112, 150.0, 7), 20, 6), 10.0, "popo")]:
        a = port.fill_pits(z, one(z), cell, bc, 1e-4)
        b = port.fill_pits_index_ties(z, one(z), cell, bc, 1e-4)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
