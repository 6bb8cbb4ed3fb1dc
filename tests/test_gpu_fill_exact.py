"""The epsilon fill on the GPU bit for bit against the oracle's restatement
of the reference's priority flood (tests/test_oracle_vs_reference.py holds
that restatement bit-equal to the compiled reference).

Surfaces: the LEM configuration's noise-plus-tilt surface (one episode of
the reference's FIFO spans almost the whole grid), fractal surfaces with
pits (thousands of small episodes), periodic grids, interior nodata holes,
LEM-like inputs (an epsilon-filled surface with small erosion pits cut into
it, the situation of every step after the first) and several epsilon
steps. Bar: zero differing cells."""
import numpy as np
import pytest

from tests import surfaces

pytestmark = pytest.mark.gpu


def _eroded(z_filled, seed, frac=0.05, depth=0.01):
    """An epsilon-filled surface with a share of cells lowered by up to
    `depth`: the small fresh pits a LEM step's erosion leaves."""
    rng = np.random.default_rng(seed)
    cut = (rng.random(z_filled.shape) < frac) * rng.random(z_filled.shape) * depth
    return (z_filled - cut.astype(np.float32)).astype(np.float32)


def _cases(port):
    one = lambda z: np.ones_like(z, np.uint8)  # noqa: E731
    z1 = port.noise_tilt_surface(512, 512, 30.0, 1, 0.0, 1.0, "nnon", 0.001)
    z2 = surfaces.fractal_pits(512)
    z3 = surfaces.fractal_pits(1024, seed=3)
    z4 = surfaces.add_pits(surfaces.fractal(160, 150, 150.0, 6), 40, 6)
    z5 = surfaces.add_pits(surfaces.fractal(96, 224, 150.0, 7), 30, 6)
    z6 = surfaces.fractal_pits(320, seed=9)
    m6 = one(z6)
    m6[100:130, 40:90] = 0
    m6[200:205, 250:300] = 0
    z1s = np.ascontiguousarray(z1[:256, :256])
    z7 = _eroded(port.fill_pits(z1s, one(z1s), 30.0, "nnon", 1e-4), 11)
    z2s = np.ascontiguousarray(z2[:384, :384])
    z8 = _eroded(port.fill_pits(z2s, one(z2s), 10.0, "oooo", 1e-4), 12, 0.1, 0.05)
    return [
        ("noise_tilt_512_nnon", z1, one(z1), 30.0, "nnon", 1e-4),
        ("fractal_pits_512", z2, one(z2), 10.0, "oooo", 1e-4),
        ("fractal_pits_1024", z3, one(z3), 10.0, "oooo", 1e-4),
        ("fractal_popo", z4, one(z4), 10.0, "popo", 1e-4),
        ("fractal_opop", z5, one(z5), 10.0, "opop", 1e-4),
        ("fractal_holes", z6, m6, 10.0, "oooo", 1e-4),
        ("lem_like_256", z7, one(z7), 30.0, "nnon", 1e-4),
        ("lem_like_384_eps_1e-3", z8, one(z8), 10.0, "oooo", 1e-3),
        ("noise_tilt_512_eps_1e-2", z1, one(z1), 30.0, "nnon", 1e-2),
    ]


def test_fill_epsilon_bitwise(port):
    import lsdtt_gb300 as G
    bad = {}
    for name, z, m, cell, bc, eps in _cases(port):
        want = port.fill_pits(z, m, cell, bc, eps)
        got = G.fill_pits(z, m, cell, bc, eps).cpu().numpy()
        nd = int((got.view(np.uint32) != want.view(np.uint32)).sum())
        print(f"{name}: {int((want != z).sum())} raised cells, {nd} differ")
        if nd:
            bad[name] = nd
    assert not bad, bad


def test_ensemble_with_a_member_per_sm_fills_like_single_grids():
    """An ensemble with at least one member per SM leaves the windows the
    small replay size cannot hold to its chains' block sweeps (fewer members
    also replay them at two larger sizes): its fill equals the single-grid
    fill bit for bit on every member, noise-plus-tilt surfaces whose long
    episodes outgrow the small size, and pitted fractals."""
    import torch
    import lsdtt_gb300 as G
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    members = []
    for k in range(sms + 8):
        if k % 4 == 3:
            z = surfaces.fractal_pits(64, seed=100 + k)
            bc = "oooo"
        else:
            z = surfaces.noise_tilt(40 + (k % 7) * 9, 48 + (k % 5) * 11, 30.0, 1000 + k, "nnon", 0.001)
            bc = "nnon"
        members.append(dict(z=z, cell_size=30.0 if bc == "nnon" else 10.0, boundary_conditions=bc,
                            fill_min_slope=1e-4, erodibility=0.0, enable_hillslope=False, uplift_rate=0.0))
    ens = G.Ensemble(members, use_graph=False)
    try:
        ens.step()
        bad = []
        for k, s in enumerate(members):
            got = ens.get(k).cpu().numpy()
            m = np.ones_like(s["z"], np.uint8)
            want = G.fill_pits(s["z"], m, s["cell_size"], s["boundary_conditions"], 1e-4).cpu().numpy()
            if not np.array_equal(got.view(np.uint32), want.view(np.uint32)):
                bad.append(k)
        assert not bad, bad
    finally:
        ens.close()
