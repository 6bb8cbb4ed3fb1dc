"""Size-independent properties of the routing outputs (epsilon fill, D8
receivers, donors, outlets, topological order, s-vector, counts and area)
for a fully valid grid with open edges ("oooo").

Each property holds for the reference's own outputs: tests/test_oracle_pins.py
checks them on the oracle (bit-equal to the reference on its pins), and the
GPU test applies them at the routing workload's full size (8192 x 8192),
where the oracle is too slow to run inside a test. Conventions follow the
reference's flowinfo (src/core/flowinfo_cpu.cpp): outlets hold receiver -2
and direction 255; direction d steps (dr, dc) below; the Kahn order
(:1428-1522) lists donors before their receiver; the s-vector (:1544-1731)
lists receivers first, start[c] is c's position and [start, start + size)
spans c's upstream cells."""
import numpy as np

D8_DR = np.array([-1, -1, 0, 1, 1, 1, 0, -1], np.int64)  # N, NE, E, SE, S, SW, W, NW
D8_DC = np.array([0, 1, 1, 1, 0, -1, -1, -1], np.int64)


def check_fill(z, filled):
    """Never lowered, open-edge seeds untouched, and every interior cell
    strictly above its lowest neighbour (min_slope > 0 leaves no flat and
    no pit)."""
    assert filled.shape == z.shape and filled.dtype == np.float32
    assert np.all(filled >= z)
    for edge in (np.s_[0, :], np.s_[-1, :], np.s_[:, 0], np.s_[:, -1]):
        assert np.array_equal(filled[edge].view(np.uint32), z[edge].view(np.uint32))
    nr, nc = filled.shape
    inner = filled[1:-1, 1:-1]
    lowest = np.full(inner.shape, np.inf, np.float32)
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            if dy or dx:
                np.minimum(lowest, filled[1 + dy:nr - 1 + dy, 1 + dx:nc - 1 + dx], out=lowest)
    assert np.all(inner > lowest)


def check_flow(filled, cell, rec, direction, donors, outlets, topo, svec, start, size, area):
    """Receivers, donors, outlets, Kahn order, s-vector, counts and area of
    one D8 build over `filled` (all cells valid, open edges)."""
    nr, nc = filled.shape
    n = nr * nc
    idx = np.arange(n, dtype=np.int64)
    f = filled.reshape(-1)
    size = size.astype(np.int64)
    # Outlets: exactly the cells without a receiver; after the fill these
    # are the edge cells.
    out = rec < 0
    assert np.all(rec[out] == -2) and np.all(direction[out] == 255)
    assert np.array_equal(np.sort(outlets), idx[out])
    assert not np.any(out.reshape(nr, nc)[1:-1, 1:-1])
    # Receivers: the D8 neighbour in the stored direction, strictly lower.
    ok = ~out
    d = direction[ok].astype(np.int64)
    assert np.all(d < 8)
    r, c = idx[ok] // nc, idx[ok] % nc
    assert np.array_equal(rec[ok], (r + D8_DR[d]) * nc + (c + D8_DC[d]))
    assert np.all(f[rec[ok]] < f[ok])
    # Donor counts.
    assert np.array_equal(donors.astype(np.int64), np.bincount(rec[ok], minlength=n))
    # Kahn order: a permutation, every donor before its receiver.
    assert topo.size == n
    pos = np.full(n, -1, np.int64)
    pos[topo] = idx
    assert np.all(pos >= 0)
    assert np.all(pos[idx[ok]] < pos[rec[ok]])
    # s-vector: a permutation, start = position, receivers first, nested
    # upstream ranges.
    assert svec.size == n
    spos = np.full(n, -1, np.int64)
    spos[svec] = idx
    assert np.all(spos >= 0)
    assert np.array_equal(start, spos)
    assert np.all(start[rec[ok]] < start[ok])
    assert np.all(start[ok] + size[ok] <= start[rec[ok]] + size[rec[ok]])
    # Counts: one plus the donors' counts (int64, exact), summing to the
    # cell count over the outlets; area = count * cell^2 in FP64 (exact when
    # cell^2 is an integer, as for the 10 m cells used here).
    up = np.bincount(rec[ok], weights=size[ok].astype(np.float64), minlength=n)
    assert np.array_equal(size, 1 + up.astype(np.int64))
    assert int(size[out].sum()) == n
    assert np.array_equal(area, size.astype(np.float64) * (cell * cell))
