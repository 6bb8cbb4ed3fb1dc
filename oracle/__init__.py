"""CPU oracle for the landscape-evolution hot path -- TEST INFRASTRUCTURE ONLY.

Two libraries sit behind this module:

* ``port``: oracle/liblsdtt_oracle.so, a C++ restatement of the reference
  algorithms (oracle/lsdtt_oracle.cpp). It builds on any host with g++ and is
  the checker the GPU parity tests and the CPU baseline use.
* ``ref``: oracle/_ref/liblsdtt_ref.so, the reference's own C++ sources
  compiled where they lie plus a thin C shim (oracle/ref_shim.cpp). It exists
  only where the reference checkout exists and is used to pin ``port``.

Only tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this package. The product (lsdtt_gb300) never does.
"""
from __future__ import annotations

import ctypes
import os
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_PATH = os.path.join(HERE, "liblsdtt_oracle.so")
REF_PATH = os.path.join(HERE, "_ref", "liblsdtt_ref.so")

_c_f32 = ctypes.POINTER(ctypes.c_float)
_c_f64 = ctypes.POINTER(ctypes.c_double)
_c_u8 = ctypes.POINTER(ctypes.c_uint8)
_c_i32 = ctypes.POINTER(ctypes.c_int32)
_c_i64 = ctypes.POINTER(ctypes.c_int64)
_c_u64 = ctypes.POINTER(ctypes.c_uint64)


def _p(a, t):
    return None if a is None else a.ctypes.data_as(t)


class OracleError(RuntimeError):
    """The oracle (restated or reference) raised; message is the reference's."""


class _Lib:
    """ctypes view of one oracle library. Both expose the same entry points
    with a ``ref_`` or ``oracle_`` prefix."""

    def __init__(self, path: str, prefix: str):
        mode = os.RTLD_LAZY if prefix == "ref_" else ctypes.DEFAULT_MODE
        self.lib = ctypes.CDLL(path, mode=mode)
        self.prefix = prefix
        self.path = path

    def fn(self, name):
        return getattr(self.lib, self.prefix + name)

    # --------------------------------------------------------------- fill
    def fill_pits(self, z, mask, cell, bc="oooo", min_slope=1e-4, nodata=-9999.0,
                  radix_queue=False):
        z = np.ascontiguousarray(z, dtype=np.float32)
        mask = np.ascontiguousarray(mask, dtype=np.uint8)
        nr, nc = z.shape
        out = np.empty_like(z)
        err = ctypes.create_string_buffer(1024)
        f = self.fn("fill_pits")
        f.restype = ctypes.c_int
        rc = f(_p(z, _c_f32), _p(mask, _c_u8), ctypes.c_int(nr), ctypes.c_int(nc),
               ctypes.c_double(cell), ctypes.c_double(nodata), bc.encode(),
               ctypes.c_float(min_slope), ctypes.c_int(int(radix_queue)),
               _p(out, _c_f32), err, ctypes.c_int(1024))
        if rc != 0:
            raise OracleError(err.value.decode())
        return out

    def fill_pits_index_ties(self, z, mask, cell, bc="oooo", min_slope=1e-4, nodata=-9999.0):
        """The priority flood with heap entries of equal value taken in
        (row, col) order (the oracle only; the reference's heap orders them
        by its layout). The GPU fill follows this rule."""
        z = np.ascontiguousarray(z, dtype=np.float32)
        mask = np.ascontiguousarray(mask, dtype=np.uint8)
        nr, nc = z.shape
        out = np.empty_like(z)
        err = ctypes.create_string_buffer(1024)
        f = self.fn("fill_pits_index_ties")
        f.restype = ctypes.c_int
        rc = f(_p(z, _c_f32), _p(mask, _c_u8), ctypes.c_int(nr), ctypes.c_int(nc),
               ctypes.c_double(cell), ctypes.c_double(nodata), bc.encode(),
               ctypes.c_float(min_slope), _p(out, _c_f32), err, ctypes.c_int(1024))
        if rc != 0:
            raise OracleError(err.value.decode())
        return out

    # --------------------------------------------------------------- D8 engine
    def flowinfo(self, z, mask, cell, bc="oooo", interior_nodata_is_outlet=True,
                 allow_pits_as_outlets=False, build_topo=True, build_sv=True,
                 require_acyclic=True, forced=None, n_threads=0, nodata=-9999.0,
                 weights=None, want_accum=True):
        z = np.ascontiguousarray(z, dtype=np.float32)
        mask = np.ascontiguousarray(mask, dtype=np.uint8)
        nr, nc = z.shape
        n = nr * nc
        rec = np.empty(n, np.int64)
        dr = np.empty(n, np.uint8)
        don = np.empty(n, np.uint8)
        outs = np.empty(max(n, 1), np.int64)
        n_out = np.zeros(1, np.int64)
        topo = np.empty(max(n, 1), np.int64)
        n_topo = np.zeros(1, np.int64)
        sv = np.empty(max(n, 1), np.int64)
        st = np.empty(n, np.int64)
        sz = np.empty(n, np.uint64)
        flags = np.zeros(2, np.int32)
        forced = np.ascontiguousarray(forced if forced is not None else [], dtype=np.int64)
        w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
        acc = np.empty(n, np.float64) if want_accum else None
        err = ctypes.create_string_buffer(1024)
        f = self.fn("flowinfo")
        f.restype = ctypes.c_int
        rc = f(_p(z, _c_f32), _p(mask, _c_u8), ctypes.c_int(nr), ctypes.c_int(nc),
               ctypes.c_double(cell), ctypes.c_double(nodata), bc.encode(),
               ctypes.c_int(int(interior_nodata_is_outlet)),
               ctypes.c_int(int(allow_pits_as_outlets)), ctypes.c_int(int(build_topo)),
               ctypes.c_int(int(build_sv)), ctypes.c_int(int(require_acyclic)),
               _p(forced, _c_i64), ctypes.c_int64(forced.size), ctypes.c_int(n_threads),
               _p(rec, _c_i64), _p(dr, _c_u8), _p(don, _c_u8), _p(outs, _c_i64),
               _p(n_out, _c_i64), _p(topo, _c_i64), _p(n_topo, _c_i64), _p(sv, _c_i64),
               _p(st, _c_i64), _p(sz, _c_u64), _p(flags, _c_i32), _p(w, _c_f64),
               _p(acc, _c_f64), err, ctypes.c_int(1024))
        if rc != 0:
            raise OracleError(err.value.decode())
        res = dict(receiver=rec, direction=dr, donors=don, outlets=outs[: n_out[0]].copy(),
                   has_topo=bool(flags[0]), has_sv=bool(flags[1]))
        if flags[0]:
            res["topo"] = topo[: n_topo[0]].copy()
            if want_accum:
                res["accum"] = acc
        if flags[1]:
            res["s_vector"] = sv[: int(mask.astype(bool).sum())].copy()
            res["sv_start"] = st
            res["sv_size"] = sz
        return res

    # --------------------------------------------------------------- query rasters
    QUERY_KINDS = {"distance_from_outlet": 0, "height_above_channel": 1, "height_above_channel_mask": 2,
                   "distance_to_channel": 3, "height_to_farthest_ridge": 4, "distance_to_farthest_ridge": 5,
                   "downstream_path_sum": 6, "upslope_sum": 7, "upslope_mean": 8}

    def flow_query(self, kind, z, mask, cell, bc="oooo", values=None, vmask=None, cmask=None, threshold=1,
                   include_self=True, nodata=-9999.0):
        """One lsdtt_flow_base query raster on the flow object of z (pits
        as outlets): returns (data float32, mask uint8, donor int64 or
        None)."""
        z = np.ascontiguousarray(z, dtype=np.float32)
        mask = np.ascontiguousarray(mask, dtype=np.uint8)
        nr, nc = z.shape
        v = None if values is None else np.ascontiguousarray(values, dtype=np.float32)
        vm = None if vmask is None else np.ascontiguousarray(vmask, dtype=np.uint8)
        cm = None if cmask is None else np.ascontiguousarray(cmask, dtype=np.uint8)
        k = self.QUERY_KINDS[kind]
        if self.prefix == "oracle_":
            v = z if v is None else v
            vm = mask if vm is None else vm
            cm = np.zeros_like(mask) if cm is None else cm
        out = np.empty_like(z)
        om = np.empty_like(mask)
        donor = np.empty(z.size, np.int64) if k == 2 else None
        err = ctypes.create_string_buffer(1024)
        f = self.fn("flow_query")
        f.restype = ctypes.c_int
        rc = f(_p(z, _c_f32), _p(mask, _c_u8), ctypes.c_int(nr), ctypes.c_int(nc), ctypes.c_double(cell),
               ctypes.c_double(nodata), bc.encode(), ctypes.c_int(k), _p(v, _c_f32), _p(vm, _c_u8), _p(cm, _c_u8),
               ctypes.c_int(threshold), ctypes.c_int(int(include_self)), _p(out, _c_f32), _p(om, _c_u8),
               _p(donor, _c_i64), err, ctypes.c_int(1024))
        if rc != 0:
            raise OracleError(err.value.decode())
        return out, om, donor

    # --------------------------------------------------------------- D-infinity
    def dinf_graph(self, z, mask, cell, bc="oooo", interior_nodata_is_outlet=True, nodata=-9999.0):
        """The D-infinity lsdtt_flowgraph_cpu: dict of rec [n, 2] (-1 none),
        w [n, 2], nrec, slope, bearing, donors, topo."""
        z = np.ascontiguousarray(z, dtype=np.float32)
        mask = np.ascontiguousarray(mask, dtype=np.uint8)
        nr, nc = z.shape
        n = z.size
        rec = np.empty(2 * n, np.int64)
        w = np.empty(2 * n, np.float32)
        nrec = np.empty(n, np.uint8)
        slope = np.empty(n, np.float32)
        bearing = np.empty(n, np.float32)
        donors = np.empty(n, np.uint8)
        topo = np.empty(n, np.int64)
        nt = np.zeros(1, np.int64)
        err = ctypes.create_string_buffer(1024)
        f = self.fn("dinf_graph")
        f.restype = ctypes.c_int
        rc = f(_p(z, _c_f32), _p(mask, _c_u8), ctypes.c_int(nr), ctypes.c_int(nc), ctypes.c_double(cell),
               ctypes.c_double(nodata), bc.encode(), ctypes.c_int(int(interior_nodata_is_outlet)), _p(rec, _c_i64),
               _p(w, _c_f32), _p(nrec, _c_u8), _p(slope, _c_f32), _p(bearing, _c_f32), _p(donors, _c_u8),
               _p(topo, _c_i64), _p(nt, _c_i64), err, ctypes.c_int(1024))
        if rc != 0:
            raise OracleError(err.value.decode())
        return dict(rec=rec.reshape(n, 2), w=w.reshape(n, 2), nrec=nrec, slope=slope, bearing=bearing,
                    donors=donors, topo=topo[:nt[0]].copy())

    def dinf_accumulate(self, z, mask, cell, bc="oooo", weights=None, nodata=-9999.0):
        z = np.ascontiguousarray(z, dtype=np.float32)
        mask = np.ascontiguousarray(mask, dtype=np.uint8)
        nr, nc = z.shape
        w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
        out = np.empty(z.size, np.float64)
        err = ctypes.create_string_buffer(1024)
        f = self.fn("dinf_accumulate")
        f.restype = ctypes.c_int
        rc = f(_p(z, _c_f32), _p(mask, _c_u8), ctypes.c_int(nr), ctypes.c_int(nc), ctypes.c_double(cell),
               ctypes.c_double(nodata), bc.encode(), _p(w, _c_f64), _p(out, _c_f64), err, ctypes.c_int(1024))
        if rc != 0:
            raise OracleError(err.value.decode())
        return out

    def dinf_stream_power(self, z, mask, cell, bc, K, m, n, dt, threshold_area=0.0, divide_area_by_dx=True,
                          slope_clamp=1e-5, nodata=-9999.0):
        z = np.ascontiguousarray(z, dtype=np.float32)
        mask = np.ascontiguousarray(mask, dtype=np.uint8)
        nr, nc = z.shape
        out = np.empty_like(z)
        err = ctypes.create_string_buffer(1024)
        f = self.fn("dinf_stream_power")
        f.restype = ctypes.c_int
        rc = f(_p(z, _c_f32), _p(mask, _c_u8), ctypes.c_int(nr), ctypes.c_int(nc), ctypes.c_double(cell),
               ctypes.c_double(nodata), bc.encode(), ctypes.c_float(K), ctypes.c_float(m), ctypes.c_float(n),
               ctypes.c_float(dt), ctypes.c_float(threshold_area), ctypes.c_int(int(divide_area_by_dx)),
               ctypes.c_float(slope_clamp), _p(out, _c_f32), err, ctypes.c_int(1024))
        if rc != 0:
            raise OracleError(err.value.decode())
        return out

    # --------------------------------------------------------------- stream power
    def stream_power(self, z, mask, cell, bc, K, m, n, dt, threshold_area=0.0,
                     divide_area_by_dx=True, slope_clamp=1e-5, k_field=None,
                     nodata=-9999.0):
        z = np.ascontiguousarray(z, dtype=np.float32)
        mask = np.ascontiguousarray(mask, dtype=np.uint8)
        nr, nc = z.shape
        out = np.empty_like(z)
        kf = None if k_field is None else np.ascontiguousarray(k_field, dtype=np.float32)
        err = ctypes.create_string_buffer(1024)
        f = self.fn("stream_power")
        f.restype = ctypes.c_int
        rc = f(_p(z, _c_f32), _p(mask, _c_u8), ctypes.c_int(nr), ctypes.c_int(nc),
               ctypes.c_double(cell), ctypes.c_double(nodata), bc.encode(),
               ctypes.c_float(K), ctypes.c_float(m), ctypes.c_float(n), ctypes.c_float(dt),
               ctypes.c_float(threshold_area), ctypes.c_int(int(divide_area_by_dx)),
               ctypes.c_float(slope_clamp), _p(kf, _c_f32), _p(out, _c_f32), err,
               ctypes.c_int(1024))
        if rc != 0:
            raise OracleError(err.value.decode())
        return out

    # --------------------------------------------------------------- LEM pieces
    def boundary_flats(self, mask, bc):
        mask = np.ascontiguousarray(mask, dtype=np.uint8)
        nr, nc = mask.shape
        out = np.empty(nr * nc, np.int64)
        f = self.fn("boundary_flats")
        f.restype = ctypes.c_int64
        k = f(_p(mask, _c_u8), ctypes.c_int(nr), ctypes.c_int(nc), bc.encode(),
              _p(out, _c_i64))
        return out[:k].copy()

    def lem_step_fluvial(self, z, mask, cell, bc, dt, K, m, n, U, boundary_flats,
                         nodata=-9999.0):
        z = np.ascontiguousarray(z, dtype=np.float32)
        mask = np.ascontiguousarray(mask, dtype=np.uint8)
        nr, nc = z.shape
        bf = np.ascontiguousarray(boundary_flats, dtype=np.int64)
        out = np.empty_like(z)
        stats = np.zeros(6, np.float32)
        err = ctypes.create_string_buffer(1024)
        f = self.fn("lem_step_fluvial")
        f.restype = ctypes.c_int
        rc = f(_p(z, _c_f32), _p(mask, _c_u8), ctypes.c_int(nr), ctypes.c_int(nc),
               ctypes.c_double(cell), ctypes.c_double(nodata), bc.encode(),
               ctypes.c_float(dt), ctypes.c_float(K), ctypes.c_float(m), ctypes.c_float(n),
               ctypes.c_float(U), _p(bf, _c_i64), ctypes.c_int64(bf.size), _p(out, _c_f32),
               _p(stats, _c_f32), err, ctypes.c_int(1024))
        if rc != 0:
            raise OracleError(err.value.decode())
        return out, stats

    def noise_tilt_surface(self, nr, nc, cell, seed, lo, hi, bc, slope):
        out = np.empty((nr, nc), np.float32)
        err = ctypes.create_string_buffer(1024)
        f = self.fn("noise_tilt_surface")
        f.restype = ctypes.c_int
        rc = f(ctypes.c_int(nr), ctypes.c_int(nc), ctypes.c_double(cell), ctypes.c_int(seed),
               ctypes.c_double(lo), ctypes.c_double(hi), bc.encode(), ctypes.c_float(slope),
               _p(out, _c_f32), err, ctypes.c_int(1024))
        if rc != 0:
            raise OracleError(err.value.decode())
        return out


_port = None
_ref = None


def port() -> _Lib:
    """The C++ restatement (builds with `make -C oracle`)."""
    global _port
    if _port is None:
        if not os.path.exists(PORT_PATH):
            raise FileNotFoundError(f"{PORT_PATH} missing: run `make -C oracle`")
        _port = _Lib(PORT_PATH, "oracle_")
    return _port


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref() -> _Lib:
    """The reference's own sources compiled (`make -C oracle ref`)."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_PATH):
            raise FileNotFoundError(f"{REF_PATH} missing: run `make -C oracle ref`")
        _ref = _Lib(REF_PATH, "ref_")
    return _ref


def fill_traced(z, mask, cell, bc="oooo", min_slope=1e-4, nodata=-9999.0):
    """Restated fill that also returns, per cell, the flat index of the cell
    whose processing queued it (-1 for seeds, -2 for nodata), its position in
    the processing sequence, and whether it was raised (went through the FIFO)."""
    lib = port().lib
    z = np.ascontiguousarray(z, dtype=np.float32)
    mask = np.ascontiguousarray(mask, dtype=np.uint8)
    nr, nc = z.shape
    out = np.empty_like(z)
    disc = np.empty(nr * nc, np.int64)
    order = np.empty(nr * nc, np.int64)
    via = np.zeros(nr * nc, np.uint8)
    err = ctypes.create_string_buffer(1024)
    f = lib.oracle_fill_pits_traced
    f.restype = ctypes.c_int
    rc = f(_p(z, _c_f32), _p(mask, _c_u8), ctypes.c_int(nr), ctypes.c_int(nc),
           ctypes.c_double(cell), ctypes.c_double(nodata), bc.encode(),
           ctypes.c_float(min_slope), _p(out, _c_f32), _p(disc, _c_i64), _p(order, _c_i64),
           _p(via, _c_u8), err, ctypes.c_int(1024))
    if rc != 0:
        raise OracleError(err.value.decode())
    return out, disc, order, via


def lem_finish(z, z_before, mask, U, dt, boundary_flats, baselevel_fall=0.0):
    """End of run_lem_step: uplift, boundary restore, statistics. Returns
    (z_out, stats[6])."""
    lib = port().lib
    z = np.array(z, dtype=np.float32, copy=True, order="C")
    zb = np.ascontiguousarray(z_before, dtype=np.float32)
    mask = np.ascontiguousarray(mask, dtype=np.uint8)
    bf = np.ascontiguousarray(boundary_flats, dtype=np.int64)
    stats = np.zeros(6, np.float32)
    f = lib.oracle_lem_finish
    f.restype = None
    f(_p(z, _c_f32), _p(zb, _c_f32), _p(mask, _c_u8), ctypes.c_int64(z.size), ctypes.c_float(U),
      ctypes.c_float(dt), ctypes.c_float(baselevel_fall), _p(bf, _c_i64), ctypes.c_int64(bf.size),
      _p(stats, _c_f32))
    return z, stats
