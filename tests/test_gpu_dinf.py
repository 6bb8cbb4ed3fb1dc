"""The D-infinity flow graph and D-infinity stream power on the GPU
(lsdtt_gpu_dinf_*) against the oracle's restatement of lsdtt_flowgraph_cpu
(method d_infinity) and compute_dinf_stream_power_incision, which
tests/test_oracle_vs_reference.py holds bit-equal to the compiled reference.

Bars: receivers, receiver counts, donor counts and the topological order
bit-exact; weights, facet slopes and bearings bit-exact except where the
in-facet angle rounds differently (the reference's atan2f against the
double atan2 rounded to float: counted, at most a few cells); accumulate
and the stream-power surface bit-exact where the weights agree, and within
1e-5 relative everywhere (the FP64 pow of the Newton iteration is the
library's on each side)."""
import numpy as np
import pytest

from tests import surfaces

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5


def _cases(port):
    z1 = port.noise_tilt_surface(160, 208, 30.0, 4, 0.0, 1.0, "nnon", 0.001)
    z2 = surfaces.fractal_pits(192, seed=5)
    m2 = np.ones_like(z2, np.uint8)
    m2[50:60, 70:95] = 0
    z3 = surfaces.add_pits(surfaces.fractal(144, 176, 150.0, 6), 30, 6)
    one = lambda z: np.ones_like(z, np.uint8)  # noqa: E731
    return [("noise_tilt_nnon", z1, one(z1), 30.0, "nnon"), ("fractal_holes_oooo", z2, m2, 10.0, "oooo"),
            ("fractal_popo", z3, one(z3), 10.0, "popo")]


def test_dinf_graph_accumulate_and_stream_power(port):
    import lsdtt_gb300 as G
    for name, z, m, cell, bc in _cases(port):
        f = port.fill_pits(z, m, cell, bc, 1e-4)
        want = port.dinf_graph(f, m, cell, bc)
        g = G.FlowGraphDinf(f, m, cell, bc)
        rec = g.receivers().cpu().numpy()
        nrec = g.n_receivers().cpu().numpy()
        assert np.array_equal(rec, want["rec"]), (name, int((rec != want["rec"]).sum()))
        assert np.array_equal(nrec, want["nrec"]), name
        assert np.array_equal(g.donor_count().cpu().numpy(), want["donors"]), name
        topo = g.topological_order().cpu().numpy()
        assert np.array_equal(topo, want["topo"]), (name, topo.size, want["topo"].size)
        w = g.weights().cpu().numpy()
        wdiff = int((w.view(np.uint32) != want["w"].view(np.uint32)).sum())
        sdiff = int((g.slopes().cpu().numpy().view(np.uint32) != want["slope"].view(np.uint32)).sum())
        bdiff = int((g.bearings().cpu().numpy().view(np.uint32) != want["bearing"].view(np.uint32)).sum())
        acc = g.accumulate().cpu().numpy()
        acc_w = port.dinf_accumulate(f, m, cell, bc)
        adiff = int((acc.view(np.uint64) != acc_w.view(np.uint64)).sum())
        arel = float(np.max(np.abs(acc - acc_w) / np.maximum(np.abs(acc_w), 1.0)))
        line = [f"{name}: weights differ in {wdiff}, slopes {sdiff}, bearings {bdiff}; accumulate {adiff} cells "
                f"(max rel {arel:.2e})"]
        assert wdiff <= 8 and sdiff <= 8 and bdiff <= 8
        assert arel < 1e-12
        if wdiff == 0:
            assert adiff == 0
        for n_exp in (1.0, 1.5, 2.0):
            got = g.stream_power(2e-5, 0.45, n_exp, 500.0).cpu().numpy()
            sp = port.dinf_stream_power(f, m, cell, bc, 2e-5, 0.45, n_exp, 500.0)
            nd = int((got.view(np.uint32) != sp.view(np.uint32)).sum())
            rel = float(np.max(np.abs(got.astype(np.float64) - sp) / np.maximum(np.abs(sp), 1.0)))
            line.append(f"SP n={n_exp}: {nd} cells differ, max rel {rel:.2e}")
            assert rel < REL_TOL, (name, n_exp, rel)
        print("; ".join(line))
        g.close()
