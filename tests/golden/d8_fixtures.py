"""The 17 hermetic D8 fixtures and option configurations of the reference's
byte-identity test (tests/cpp/test_flow_d8_identity.cpp:144-338), restated,
plus the FNV-1a hashing it pins (:117-131, 343-420).

Every elevation is an integer: z = 1000*d + noise with noise in
{0, 250, 500, 750}, d the BFS step distance (under the router's own boundary
rules) to the nearest cell that may drain out, and all randomness from the
64-bit LCG s = s*6364136223846793005 + 1442695040888963407, output s >> 33.
"""
from __future__ import annotations

from collections import deque

import numpy as np

MASK64 = (1 << 64) - 1
D8_ROW = (-1, -1, 0, 1, 1, 1, 0, -1)
D8_COL = (0, 1, 1, 1, 0, -1, -1, -1)
ABSENT = 0xABAD1DEAABAD1DEA

# name, rows, cols, cell, bc, mask kind, interior_nodata_is_outlet, n_forced, pits_as_outlets, seed
SPECS = [
    ("open_square", 61, 67, 10.0, "oooo", "none", True, 0, False, 11),
    ("open_nonint_cell", 47, 53, 30.137, "oooo", "none", True, 0, False, 12),
    ("holes_nodata_outlet", 59, 71, 10.0, "oooo", "holes", True, 0, False, 13),
    ("holes_nodata_blocked", 59, 71, 10.0, "oooo", "holes", False, 0, False, 14),
    ("nodata_border", 43, 57, 10.0, "oooo", "border", True, 0, False, 15),
    ("noflux_forced", 41, 45, 10.0, "nnnn", "none", True, 6, False, 16),
    ("periodic_forced", 37, 39, 10.0, "pppp", "none", True, 4, False, 17),
    ("periodic_ns_open_ew", 35, 41, 10.0, "popo", "none", True, 0, False, 18),
    ("baselevel_edges", 33, 36, 10.0, "bbbb", "none", True, 0, False, 19),
    ("mixed_onbn", 38, 44, 10.0, "onbn", "holes", True, 0, False, 20),
    ("forced_on_open", 40, 40, 10.0, "oooo", "none", True, 5, False, 21),
    ("pits_as_outlets", 31, 37, 10.0, "nnnn", "none", True, 0, True, 22),
    ("periodic_2_rows", 2, 9, 10.0, "pppp", "none", True, 1, False, 23),
    ("periodic_1_col", 7, 1, 10.0, "pppp", "none", True, 1, False, 24),
    ("tiny_3x3_periodic", 3, 3, 10.0, "pppp", "none", True, 1, False, 25),
    ("single_cell", 1, 1, 10.0, "oooo", "none", True, 0, False, 26),
    ("two_by_n", 2, 11, 10.0, "oooo", "none", True, 0, False, 27),
]

# name, keep topological order, build s-vector, require acyclic
CONFIGS = [
    ("sv_on", True, True, True),
    ("sv_off", True, False, True),
    ("sv_only", False, True, True),
    ("receivers_only", False, False, False),
]


class _Lcg:
    def __init__(self, seed: int):
        self.s = seed & MASK64

    def __call__(self) -> int:
        self.s = (self.s * 6364136223846793005 + 1442695040888963407) & MASK64
        return self.s >> 33


def _step(bc, nr, nc, row, col, d):
    """Router neighbour rule: None = blocked, 'off' = leaves via o/b edge."""
    r, c = row + D8_ROW[d], col + D8_COL[d]
    off = False

    def edge(b, wrap):
        nonlocal off
        if b == "p":
            return True, wrap
        if b in "ob":
            off = True
            return True, None
        return False, None

    if r < 0:
        ok, w = edge(bc[0], nr - 1)
        if not ok:
            return None
        r = w if w is not None else r
    if r >= nr:
        ok, w = edge(bc[2], 0)
        if not ok:
            return None
        r = w if w is not None else r
    if c < 0:
        ok, w = edge(bc[3], nc - 1)
        if not ok:
            return None
        c = w if w is not None else c
    if c >= nc:
        ok, w = edge(bc[1], 0)
        if not ok:
            return None
        c = w if w is not None else c
    if off:
        return "off"
    return r, c


def make_fixture(spec):
    """Returns dict(z float32[nr,nc], mask u8[nr,nc], forced int64[], cell, bc, ...)."""
    name, nr, nc, cell, bc, mkind, nd_out, n_forced, pits, seed = spec
    n = nr * nc
    rng = _Lcg(seed)
    m = np.ones(n, np.uint8)
    for r in range(nr):
        for c in range(nc):
            i = r * nc + c
            if mkind == "holes" and rng() % 100 < 4:
                m[i] = 0
            if mkind == "border" and (r < 2 or c < 3 or r >= nr - 1):
                m[i] = 0
    forced = []
    for _ in range(n_forced):
        f = rng() % n
        while m[f] == 0:
            f = (f + 1) % n
        if f not in forced:
            forced.append(f)
    dist = np.full(n, -1, np.int64)
    q = deque()
    for r in range(nr):
        for c in range(nc):
            i = r * nc + c
            if not m[i]:
                continue
            sink = i in forced
            if (r == 0 and bc[0] == "b") or (c == nc - 1 and bc[1] == "b") or \
               (r == nr - 1 and bc[2] == "b") or (c == 0 and bc[3] == "b"):
                sink = True
            d = 0
            while d < 8 and not sink:
                s = _step(bc, nr, nc, r, c, d)
                d += 1
                if s is None:
                    continue
                if s == "off":
                    sink = True
                    break
                if not m[s[0] * nc + s[1]] and nd_out:
                    sink = True
            if sink:
                dist[i] = 0
                q.append(i)
    while q:
        i = q.popleft()
        r, c = divmod(i, nc)
        for d in range(8):
            s = _step(bc, nr, nc, r, c, d)
            if s is None or s == "off":
                continue
            j = s[0] * nc + s[1]
            if not m[j] or dist[j] >= 0:
                continue
            dist[j] = dist[i] + 1
            q.append(j)
    z = np.full(n, -9999.0, np.float32)
    for i in range(n):
        if not m[i]:
            continue
        noise = (rng() % 4) * 250
        if pits:
            zz = 1000 + noise
        else:
            if dist[i] < 0:
                raise ValueError(f"fixture {name} has a cell with no route out")
            zz = 1000 * int(dist[i]) + noise
        z[i] = float(zz)
    return dict(name=name, z=z.reshape(nr, nc), mask=m.reshape(nr, nc), forced=np.array(forced, np.int64),
                cell=cell, bc=bc, interior_nodata_is_outlet=nd_out, pits_as_outlets=pits)


class Fnv64:
    def __init__(self):
        self.h = 1469598103934665603

    def bytes(self, b: bytes):
        h = self.h
        for x in b:
            h = ((h ^ x) * 1099511628211) & MASK64
        self.h = h

    def vec(self, arr: np.ndarray):
        self.bytes(np.uint64(arr.size).tobytes())
        if arr.size:
            self.bytes(np.ascontiguousarray(arr).tobytes())


def hash_components(fx, res) -> dict:
    """Hash a flow result dict (receiver, direction, donors, outlets, topo,
    s_vector, sv_start, sv_size, has_topo, has_sv, accum_w) the way the
    reference test does. `accum_w` is accumulate() with the test's
    non-uniform weights; `area` is the drainage-area raster data+mask."""
    n = fx["z"].size
    out = {}
    interleaved = lambda *arrs: np.stack(arrs, axis=1)  # noqa: E731
    h = Fnv64(); h.bytes(np.ascontiguousarray(res["receiver"], np.int64).tobytes()); out["receiver"] = h.h
    h = Fnv64(); h.bytes(np.ascontiguousarray(res["direction"], np.uint8).tobytes()); out["direction"] = h.h
    h = Fnv64(); h.bytes(np.ascontiguousarray(res["donors"], np.uint8).tobytes()); out["donors"] = h.h
    h = Fnv64(); h.vec(np.ascontiguousarray(res["outlets"], np.int64)); out["outlets"] = h.h
    out["topo"] = ABSENT
    if res["has_topo"]:
        h = Fnv64(); h.vec(np.ascontiguousarray(res["topo"], np.int64)); out["topo"] = h.h
    out["svector"] = ABSENT
    mask = fx["mask"].ravel()
    if res["has_sv"]:
        h = Fnv64()
        sv = np.ascontiguousarray(res["s_vector"], np.int64)
        h.bytes(sv.tobytes())  # concatenated outlet slices == the s-vector
        h.bytes(np.uint64(sv.size).tobytes())
        rec = np.zeros(n, dtype=[("s", "<i8"), ("z", "<u8")])
        rec["s"] = res["sv_start"]
        rec["z"] = res["sv_size"]
        h.bytes(rec.tobytes())
        out["svector"] = h.h
    out["area"] = ABSENT
    if res["has_sv"] or res["has_topo"]:
        cell = fx["cell"]
        if res["has_sv"]:
            data = np.where(mask != 0, (res["sv_size"].astype(np.float64) * (cell * cell)).astype(np.float32),
                            np.float32(-9999.0))
        else:
            data = np.where(mask != 0, res["accum_area"].astype(np.float32), np.float32(-9999.0))
        h = Fnv64(); h.vec(data.astype(np.float32)); h.vec((mask != 0).astype(np.uint8)); out["area"] = h.h
    out["weighted"] = ABSENT
    if res["has_topo"]:
        h = Fnv64(); h.vec(np.ascontiguousarray(res["accum_w"], np.float64)); out["weighted"] = h.h
    return out


def test_weights(n: int) -> np.ndarray:
    f = np.arange(n, dtype=np.int64)
    return 0.125 + 0.375 * (f % 7).astype(np.float64)
