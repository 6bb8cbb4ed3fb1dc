"""The routing path at its workload's full size: an 8192 x 8192 fractal
(k^-2 spectrum, 1000 m relief) with 100,000 pits, dx = 10 m, epsilon 1e-4,
open edges. The outputs are checked through the size-independent properties
of tests/routing_props.py (which the oracle's own outputs satisfy), the
host-buffer C-ABI route is required to give the device path's bits, and
the epsilon fill, the epsilon-0 fill and every D8 output are compared bit
for bit with the oracle (about a minute of CPU time at this size)."""
import ctypes

import numpy as np
import pytest

from tests import routing_props as RP
from tests import surfaces

pytestmark = pytest.mark.gpu

N = 8192
CELL = 10.0


@pytest.fixture(scope="module")
def surface():
    z = surfaces.fractal_pits(N)
    return z, np.ones_like(z, np.uint8)


def test_routing_full_size_properties(surface):
    import lsdtt_gb300 as G
    z, m = surface
    filled_d = G.fill_pits(z, m, CELL, "oooo", 1e-4)
    filled = filled_d.cpu().numpy()
    RP.check_fill(z, filled)
    fi = G.FlowInfo(filled_d, m, CELL, "oooo", allow_pits_as_outlets=True)
    try:
        host = lambda t: t.cpu().numpy()  # noqa: E731
        RP.check_flow(filled, CELL, host(fi.receiver()), host(fi.direction()), host(fi.donor_count()),
                      host(fi.outlets()), host(fi.topological_order()), host(fi.s_vector()),
                      host(fi.s_vector_start()), host(fi.s_vector_size()), host(fi.accumulate()))
        rec_d, topo_d, size_d = host(fi.receiver()), host(fi.topological_order()), host(fi.s_vector_size())
    finally:
        fi.close()

    # The same route through the host-buffer entry point.
    n = z.size
    f_h = np.empty_like(z)
    rec = np.empty(n, np.int64)
    topo = np.empty(n, np.int64)
    cnt = np.empty(n, np.uint64)
    g = G.make_grid(N, N, CELL, "oooo")
    opts = G.FlowOptions(1, 1, 1, 1, 1)
    vp = lambda a: ctypes.c_void_p(a.ctypes.data)  # noqa: E731
    G._check(G.lib().lsdtt_gpu_route_host(ctypes.byref(g), vp(z), vp(m), ctypes.c_float(1e-4), ctypes.byref(opts),
                                          vp(f_h), vp(rec), vp(topo), vp(cnt), None))
    assert np.array_equal(f_h.view(np.uint32), filled.view(np.uint32))
    assert np.array_equal(rec, rec_d)
    assert np.array_equal(topo, topo_d)
    assert np.array_equal(cnt.astype(np.int64), size_d.astype(np.int64))


def test_routing_full_size_bitwise_against_oracle(surface, port):
    """The same 8192 x 8192 workload compared bit for bit with the oracle:
    the epsilon fill (against the oracle with (value, cell index) heap ties,
    the order the GPU defines where the reference's heap layout decides; the
    cells where the reference's own order differs are counted), the
    epsilon-0 fill, and every D8 output (receivers, directions, donor counts,
    outlets, Kahn order, s-vector, starts, contributing counts, drainage
    area) on that fill."""
    import time
    import lsdtt_gb300 as G
    z, m = surface
    want0 = port.fill_pits(z, m, CELL, "oooo", 0.0)
    got0 = G.fill_pits(z, m, CELL, "oooo", 0.0).cpu().numpy()
    assert np.array_equal(got0.view(np.uint32), want0.view(np.uint32))
    del want0, got0
    zd = G._dev(z, G._torch().float32)
    md = G._dev(m, G._torch().uint8)
    G.fill_pits(zd, md, CELL, "oooo", 1e-4)
    G._torch().cuda.synchronize()
    t0 = time.perf_counter()
    got = G.fill_pits(zd, md, CELL, "oooo", 1e-4)
    G._torch().cuda.synchronize()
    dt = time.perf_counter() - t0
    got = got.cpu().numpy()
    f = port.fill_pits_index_ties(z, m, CELL, "oooo", 1e-4)
    ref = port.fill_pits(z, m, CELL, "oooo", 1e-4)
    n_tie = int((ref.view(np.uint32) != f.view(np.uint32)).sum())
    print(f"epsilon fill {N}^2: {dt * 1e3:.1f} ms on the GPU, {int((f != z).sum())} raised cells, "
          f"{n_tie} differ between the reference's heap order and (value, index) ties")
    assert np.array_equal(got.view(np.uint32), f.view(np.uint32))
    del got, ref
    want = port.flowinfo(f, m, CELL, "oooo", allow_pits_as_outlets=True)
    fi = G.FlowInfo(f, m, CELL, "oooo", allow_pits_as_outlets=True)
    try:
        host = lambda t: t.cpu().numpy()  # noqa: E731
        assert np.array_equal(host(fi.receiver()), want["receiver"])
        assert np.array_equal(host(fi.direction()), want["direction"])
        assert np.array_equal(host(fi.donor_count()), want["donors"])
        assert np.array_equal(host(fi.outlets()), want["outlets"])
        assert np.array_equal(host(fi.topological_order()), want["topo"])
        assert np.array_equal(host(fi.s_vector()), want["s_vector"])
        assert np.array_equal(host(fi.s_vector_start()), want["sv_start"])
        assert np.array_equal(host(fi.s_vector_size()).astype(np.uint64), want["sv_size"])
        assert np.array_equal(host(fi.accumulate()).view(np.uint64), want["accum"].view(np.uint64))
    finally:
        fi.close()
