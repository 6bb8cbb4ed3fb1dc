"""lsdtt_gb300 -- GB300 (sm_103a) backend for the lsdtt3 landscape-evolution
timestep hot path.

This module is the Python face of the C ABI in include/lsdtt_gb300.h. It
mirrors the reference's own Python surface for the path (lsdtt3.FlowInfo,
lsdtt3.fill_pits, LandscapeModel.step; python_bindings/bindings/flow_info.cpp,
raster_pit_processing.cpp, landscape_model.cpp) with the same argument
meaning and the same error messages, and keeps every array in device memory.
PyTorch supplies device allocation and streams; all computation happens in
liblsdtt_gb300.so. There is no CPU fallback: importing works anywhere, but
every call fails loudly when the library or a CUDA device is missing.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblsdtt_gb300.so")

# status codes (include/lsdtt_gb300.h)
OK, ENODEV, ENOMEM, EINVAL, EUNRESOLVED, ECYCLIC, ENOCONV, ETIMEOUT, ECUDA, EOVERFLOW, ESTATE = range(11)


class GpuError(RuntimeError):
    """A non-zero status from the library. `status` is the C status code and
    the message is the reference's exception text where the reference throws."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


class Grid(ctypes.Structure):
    _fields_ = [("n_rows", ctypes.c_int32), ("n_cols", ctypes.c_int32), ("cell_size", ctypes.c_double),
                ("no_data_value", ctypes.c_double), ("boundary_conditions", ctypes.c_char * 4)]


class FlowOptions(ctypes.Structure):
    _fields_ = [("interior_nodata_is_outlet", ctypes.c_int32), ("require_acyclic_graph", ctypes.c_int32),
                ("build_topological_order", ctypes.c_int32), ("build_s_vector", ctypes.c_int32),
                ("allow_pits_as_outlets", ctypes.c_int32)]


class FlowView(ctypes.Structure):
    _fields_ = [("receiver", ctypes.c_void_p), ("direction", ctypes.c_void_p), ("donor_count", ctypes.c_void_p),
                ("outlets", ctypes.c_void_p), ("topological_order", ctypes.c_void_p), ("s_vector", ctypes.c_void_p),
                ("s_vector_start", ctypes.c_void_p), ("s_vector_size", ctypes.c_void_p), ("n_cells", ctypes.c_int64),
                ("n_valid_cells", ctypes.c_int64), ("n_outlets", ctypes.c_int64), ("is_acyclic", ctypes.c_int32),
                ("has_topological_order", ctypes.c_int32), ("has_s_vector", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


_lib = None


def lib() -> ctypes.CDLL:
    """The loaded liblsdtt_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m lsdtt_gb300.build`")
        L = ctypes.CDLL(LIB_PATH)
        vp, i32, i64, f32 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_float
        L.lsdtt_gpu_last_error.restype = ctypes.c_char_p
        L.lsdtt_gpu_version.restype = ctypes.c_char_p
        L.lsdtt_gpu_device_available.restype = ctypes.c_int
        for name, args in {
            "lsdtt_gpu_fill_pits": [ctypes.POINTER(Grid), vp, vp, f32, vp, vp],
            "lsdtt_gpu_flow_create": [ctypes.POINTER(Grid), ctypes.POINTER(vp)],
            "lsdtt_gpu_flow_destroy": [vp],
            "lsdtt_gpu_flow_build": [vp, vp, vp, ctypes.POINTER(FlowOptions), vp, i64, vp],
            "lsdtt_gpu_flow_get_view": [vp, ctypes.POINTER(FlowView)],
            "lsdtt_gpu_flow_accumulate": [vp, vp, vp, vp],
            "lsdtt_gpu_stream_power_d8": [vp, vp, vp, f32, f32, f32, f32, f32, i32, f32, vp, vp],
            "lsdtt_gpu_route_host": [ctypes.POINTER(Grid), vp, vp, f32, ctypes.POINTER(FlowOptions), vp, vp, vp, vp,
                                     vp],
        }.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        _lib = L
    return _lib


def _check(status: int):
    if status != OK:
        raise GpuError(status, lib().lsdtt_gpu_last_error().decode())


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise GpuError(ENODEV, "lsdtt_gb300: no CUDA device")
    return torch


def _dev(a, dtype):
    """Device tensor view/copy of a numpy array or tensor, contiguous."""
    torch = _torch()
    if isinstance(a, torch.Tensor):
        t = a.to(device="cuda", dtype=dtype)
    else:
        t = torch.from_numpy(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype)
    return t.contiguous()


def _stream(stream):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def make_grid(n_rows: int, n_cols: int, cell_size: float, boundary_conditions: str = "oooo",
              no_data_value: float = -9999.0) -> Grid:
    bc = (boundary_conditions or "")
    if len(bc) != 4:
        raise GpuError(EINVAL, "lsdtt_flowinfo: boundary_conditions must have length 4 (north, east, south, west)")
    return Grid(int(n_rows), int(n_cols), float(cell_size), float(no_data_value), bc.encode())


def fill_pits(z, mask, cell_size: float, boundary_conditions: str = "oooo", min_slope: float = 1e-4,
              no_data_value: float = -9999.0, out=None, stream=None):
    """fill_pits(raster, min_slope, bc) on the GPU. Returns a float32 CUDA
    tensor; masked/nodata cells hold no_data_value."""
    torch = _torch()
    zt = _dev(z, torch.float32)
    mt = _dev(mask, torch.uint8)
    nr, nc = zt.shape
    g = make_grid(nr, nc, cell_size, boundary_conditions, no_data_value)
    if out is None:
        out = torch.empty_like(zt)
    _check(lib().lsdtt_gpu_fill_pits(ctypes.byref(g), ctypes.c_void_p(zt.data_ptr()), ctypes.c_void_p(mt.data_ptr()),
                                     ctypes.c_float(min_slope), ctypes.c_void_p(out.data_ptr()), _stream(stream)))
    return out


class FlowInfo:
    """The D8 engine (lsdtt_flowinfo) on the GPU.

    Same constructor options as lsdtt_flowinfo_options
    (src/core/lsdtt_flow_base.hpp:79-111). Array accessors return CUDA
    tensors that stay valid until the next build() or close()."""

    def __init__(self, z, mask, cell_size: float, boundary_conditions: str = "oooo", *,
                 interior_nodata_is_outlet: bool = True, require_acyclic_graph: bool = True,
                 build_topological_order: bool = True, build_s_vector: bool = True,
                 allow_pits_as_outlets: bool = False, forced_outlet_flats: Sequence[int] = (),
                 no_data_value: float = -9999.0, stream=None):
        torch = _torch()
        zt = _dev(z, torch.float32)
        nr, nc = zt.shape
        self.shape = (nr, nc)
        self.cell_size = float(cell_size)
        self.grid = make_grid(nr, nc, cell_size, boundary_conditions, no_data_value)
        h = ctypes.c_void_p()
        _check(lib().lsdtt_gpu_flow_create(ctypes.byref(self.grid), ctypes.byref(h)))
        self._h = h
        self.options = FlowOptions(int(interior_nodata_is_outlet), int(require_acyclic_graph),
                                   int(build_topological_order), int(build_s_vector), int(allow_pits_as_outlets))
        self._forced = forced_outlet_flats
        self.build(zt, mask, stream=stream)

    def build(self, z, mask, stream=None):
        torch = _torch()
        zt = _dev(z, torch.float32)
        mt = _dev(mask, torch.uint8)
        forced = None
        nf = 0
        if self._forced is not None and len(self._forced):
            forced = _dev(np.asarray(self._forced, np.int64), torch.int64)
            nf = forced.numel()
        self._keep = (zt, mt, forced)
        _check(lib().lsdtt_gpu_flow_build(self._h, ctypes.c_void_p(zt.data_ptr()), ctypes.c_void_p(mt.data_ptr()),
                                          ctypes.byref(self.options),
                                          ctypes.c_void_p(forced.data_ptr() if forced is not None else 0),
                                          ctypes.c_int64(nf), _stream(stream)))
        v = FlowView()
        _check(lib().lsdtt_gpu_flow_get_view(self._h, ctypes.byref(v)))
        self.view = v
        return self

    # -- array views ----------------------------------------------------
    def _wrap(self, ptr, count, dtype):
        """Zero-copy CUDA tensor over an engine-owned device array."""
        torch = _torch()
        if not ptr:
            return None
        return torch.as_tensor(_DeviceArray(ptr, int(count), dtype), device="cuda")

    def receiver(self):
        return self._wrap(self.view.receiver, self.view.n_cells, _torch().int64)

    def direction(self):
        return self._wrap(self.view.direction, self.view.n_cells, _torch().uint8)

    def donor_count(self):
        return self._wrap(self.view.donor_count, self.view.n_cells, _torch().uint8)

    def outlets(self):
        return self._wrap(self.view.outlets, self.view.n_outlets, _torch().int64)

    def topological_order(self):
        if not self.view.has_topological_order:
            raise GpuError(ESTATE, "topological_order not built - set build_topological_order = true in "
                                   "lsdtt_flowinfo_options")
        return self._wrap(self.view.topological_order, self.view.n_valid_cells, _torch().int64)

    def s_vector(self):
        self._need_sv()
        return self._wrap(self.view.s_vector, self.view.n_valid_cells, _torch().int64)

    def s_vector_start(self):
        self._need_sv()
        return self._wrap(self.view.s_vector_start, self.view.n_cells, _torch().int64)

    def s_vector_size(self):
        self._need_sv()
        t = self._wrap(self.view.s_vector_size, self.view.n_cells, _torch().int64)
        return t  # uint64 counts (never above 2^63)

    def _need_sv(self):
        if not self.view.has_s_vector:
            raise GpuError(ESTATE, "s_vector not built - set build_s_vector = true in lsdtt_flowinfo_options")

    def has_topological_order(self):
        return bool(self.view.has_topological_order)

    def has_s_vector(self):
        return bool(self.view.has_s_vector)

    def n_valid_cells(self):
        return int(self.view.n_valid_cells)

    def accumulate(self, weights=None, stream=None):
        """lsdtt_flowinfo::accumulate(cell_weights): float64 CUDA tensor."""
        torch = _torch()
        out = torch.empty(self.view.n_cells, dtype=torch.float64, device="cuda")
        w = None if weights is None else _dev(weights, torch.float64).reshape(-1)
        _check(lib().lsdtt_gpu_flow_accumulate(self._h, ctypes.c_void_p(w.data_ptr() if w is not None else 0),
                                               ctypes.c_void_p(out.data_ptr()), _stream(stream)))
        return out

    # The lsdtt_flow_base query rasters (lsdtt_gpu_flow_query kinds).
    QUERY_KINDS = {"distance_from_outlet": 0, "height_above_channel": 1, "height_above_channel_mask": 2,
                   "distance_to_channel": 3, "height_to_farthest_ridge": 4, "distance_to_farthest_ridge": 5,
                   "downstream_path_sum": 6, "upslope_sum": 7, "upslope_mean": 8}

    def query(self, kind, values=None, value_mask=None, channel_mask=None, threshold=1, include_self=True,
              stream=None):
        """One query raster by name (get_<kind>_raster of lsdtt_flowinfo;
        channel_mask is the sink mask of downstream_path_sum). Returns
        (data float32, mask uint8, donor int64 or None) CUDA tensors of the
        grid's shape."""
        torch = _torch()
        k = self.QUERY_KINDS[kind]
        shape = self.shape
        vt = None if values is None else _dev(values, torch.float32).reshape(shape).contiguous()
        vm = None if value_mask is None else _dev(value_mask, torch.uint8).reshape(shape).contiguous()
        cm = None if channel_mask is None else _dev(channel_mask, torch.uint8).reshape(shape).contiguous()
        out = torch.empty(shape, dtype=torch.float32, device="cuda")
        om = torch.empty(shape, dtype=torch.uint8, device="cuda")
        donor = torch.empty(shape, dtype=torch.int64, device="cuda") if k == 2 else None
        vp = ctypes.c_void_p
        fn = lib().lsdtt_gpu_flow_query
        fn.argtypes = [vp, ctypes.c_int32, vp, vp, vp, ctypes.c_int32, ctypes.c_int32, vp, vp, vp, vp]
        fn.restype = ctypes.c_int
        ptr = lambda t: vp(t.data_ptr() if t is not None else 0)  # noqa: E731
        _check(fn(self._h, k, ptr(vt), ptr(vm), ptr(cm), int(threshold), int(bool(include_self)), ptr(out), ptr(om),
                  ptr(donor), _stream(stream)))
        return out, om, donor

    def close(self):
        if getattr(self, "_h", None):
            lib().lsdtt_gpu_flow_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _DeviceArray:
    """__cuda_array_interface__ holder for a raw device pointer."""

    _TYPESTR = {"torch.int64": "<i8", "torch.uint8": "|u1", "torch.float32": "<f4", "torch.float64": "<f8",
                "torch.int32": "<i4"}

    def __init__(self, ptr, count, dtype):
        self.__cuda_array_interface__ = {"shape": (count,), "typestr": self._TYPESTR[str(dtype)],
                                         "data": (int(ptr), False), "version": 3, "strides": None}


class SolveReport(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int32), ("converged", ctypes.c_int32), ("relative_residual", ctypes.c_double),
                ("initial_residual_inf", ctypes.c_double), ("linear_solves", ctypes.c_int32),
                ("network_applications", ctypes.c_int32), ("rejected_solves", ctypes.c_int32),
                ("fallback_iterations", ctypes.c_int32), ("explicit_relative_residual", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class LemOptions(ctypes.Structure):
    _fields_ = [("timestep", ctypes.c_float), ("erodibility", ctypes.c_float), ("m_exponent", ctypes.c_float),
                ("n_exponent", ctypes.c_float), ("uplift_rate", ctypes.c_float),
                ("hillslope_diffusivity", ctypes.c_float), ("slope_clamp", ctypes.c_float),
                ("baselevel_fall_rate", ctypes.c_float), ("fill_min_slope", ctypes.c_float),
                ("enable_hillslope", ctypes.c_int32), ("divide_area_by_dx", ctypes.c_int32),
                ("hillslope_rel_tol", ctypes.c_double), ("hillslope_max_iter", ctypes.c_int32),
                ("hillslope_nonlinear", ctypes.c_int32), ("critical_slope", ctypes.c_float)]


class LemStats(ctypes.Structure):
    _fields_ = [("delta_max_elevation", ctypes.c_float), ("delta_mean_elevation", ctypes.c_float),
                ("max_local_elevation_change", ctypes.c_float), ("p999_local_elevation_change", ctypes.c_float),
                ("mean_erosion_rate", ctypes.c_float), ("max_erosion_rate", ctypes.c_float),
                ("hillslope_iterations", ctypes.c_int32), ("reserved", ctypes.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class Member(ctypes.Structure):
    _fields_ = [("grid", Grid), ("options", LemOptions)]


class EnsembleInfo(ctypes.Structure):
    _fields_ = [("packed_cells", ctypes.c_int64), ("member_cells", ctypes.c_int64),
                ("graph_enabled", ctypes.c_int32), ("graph_captures", ctypes.c_int32),
                ("graph_replays", ctypes.c_int32), ("eager_steps", ctypes.c_int32),
                ("fill_pass_cap", ctypes.c_int32), ("depth_cap", ctypes.c_int32),
                ("sweep_split_level", ctypes.c_int32), ("sweep_block", ctypes.c_int32),
                ("hillslope_iteration_cap", ctypes.c_int32), ("last_fill_passes", ctypes.c_int32),
                ("last_max_depth", ctypes.c_int32), ("last_hillslope_iterations", ctypes.c_int32),
                ("tuned_sweep_ms", ctypes.c_double), ("untuned_sweep_ms", ctypes.c_double),
                ("sweep_dataflow", ctypes.c_int32), ("deep_members", ctypes.c_int32),
                ("dataflow_sweep_ms", ctypes.c_double), ("coop_sweep_ms", ctypes.c_double),
                ("cluster_sweep_ms", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def _bind_more():
    L = lib()
    vp, i32, f32, f64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_float, ctypes.c_double
    for name, args in {
        "lsdtt_gpu_hillslope_linear_implicit": [ctypes.POINTER(Grid), vp, vp, vp, f32, f32, f64, i32, vp,
                                                ctypes.POINTER(SolveReport), vp],
        "lsdtt_gpu_lem_create": [ctypes.POINTER(Grid), vp, ctypes.POINTER(LemOptions), ctypes.POINTER(vp), vp],
        "lsdtt_gpu_lem_destroy": [vp],
        "lsdtt_gpu_lem_step": [vp, vp, ctypes.POINTER(LemStats), vp],
        "lsdtt_gpu_ensemble_create": [ctypes.POINTER(Member), i32, i32, ctypes.POINTER(vp), vp],
        "lsdtt_gpu_ensemble_destroy": [vp],
        "lsdtt_gpu_ensemble_offsets": [vp, vp],
        "lsdtt_gpu_ensemble_set_member": [vp, i32, vp, vp, vp],
        "lsdtt_gpu_ensemble_get_member": [vp, i32, vp, vp],
        "lsdtt_gpu_ensemble_set_surface": [vp, i32, vp, vp],
        "lsdtt_gpu_ensemble_step": [vp, i32, ctypes.POINTER(LemStats), vp],
        "lsdtt_gpu_ensemble_get_info": [vp, ctypes.POINTER(EnsembleInfo)],
        "lsdtt_gpu_ensemble_override_schedule": [vp, i32, i32, i32],
        "lsdtt_gpu_ensemble_set_member_groups": [vp, i32],
        "lsdtt_gpu_ensemble_upload": [vp, vp, vp],
        "lsdtt_gpu_ensemble_download": [vp, vp, vp],
    }.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    return L


def hillslope_linear_implicit(z, mask, cell_size, boundary_conditions, D, dt, rel_tol=1e-8, max_iter=2000,
                              is_channel=None, stream=None):
    """One backward-Euler linear hillslope step (compute_hillslope_newton,
    alpha = 1). Returns (z_out CUDA tensor, SolveReport)."""
    torch = _torch()
    L = _bind_more()
    zt = _dev(z, torch.float32)
    mt = _dev(mask, torch.uint8)
    ct = None if is_channel is None else _dev(is_channel, torch.uint8)
    g = make_grid(zt.shape[0], zt.shape[1], cell_size, boundary_conditions)
    out = torch.empty_like(zt)
    rep = SolveReport()
    st = L.lsdtt_gpu_hillslope_linear_implicit(ctypes.byref(g), ctypes.c_void_p(zt.data_ptr()),
                                               ctypes.c_void_p(mt.data_ptr()),
                                               ctypes.c_void_p(ct.data_ptr() if ct is not None else 0),
                                               ctypes.c_float(D), ctypes.c_float(dt), ctypes.c_double(rel_tol),
                                               ctypes.c_int32(max_iter), ctypes.c_void_p(out.data_ptr()),
                                               ctypes.byref(rep), _stream(stream))
    _check(st)
    return out, rep


def stream_power_d8(flow: "FlowInfo", z, K, m, n, dt, incision_threshold_area=0.0, divide_area_by_dx=True,
                    slope_clamp=1e-5, erodibility_field=None, stream=None):
    """compute_d8_stream_power_incision on a built FlowInfo (moving-average
    kernel 1, no width correction). Returns a float32 CUDA tensor."""
    torch = _torch()
    zt = _dev(z, torch.float32)
    kf = None if erodibility_field is None else _dev(erodibility_field, torch.float32)
    out = torch.empty_like(zt)
    _check(lib().lsdtt_gpu_stream_power_d8(flow._h, ctypes.c_void_p(zt.data_ptr()),
                                           ctypes.c_void_p(kf.data_ptr() if kf is not None else 0),
                                           ctypes.c_float(K), ctypes.c_float(m), ctypes.c_float(n), ctypes.c_float(dt),
                                           ctypes.c_float(incision_threshold_area),
                                           ctypes.c_int32(int(divide_area_by_dx)), ctypes.c_float(slope_clamp),
                                           ctypes.c_void_p(out.data_ptr()), _stream(stream)))
    return out


class LandscapeModel:
    """Device-resident LEM (run_lem_step in the D8 coupled regime with the
    linear implicit hillslope), optionally filling the surface each step."""

    def __init__(self, z, mask, cell_size, boundary_conditions="oooo", *, timestep=100.0, erodibility=1e-3,
                 m_exponent=0.45, n_exponent=1.0, uplift_rate=1e-4, hillslope_diffusivity=1e-3,
                 enable_hillslope=True, slope_clamp=1e-5, baselevel_fall_rate=0.0, fill_min_slope=0.0,
                 divide_area_by_dx=True, hillslope_rel_tol=1e-8, hillslope_max_iter=2000, hillslope_nonlinear=False,
                 critical_slope=1.0, stream=None):
        torch = _torch()
        L = _bind_more()
        self.z = _dev(z, torch.float32).clone()
        self.mask = _dev(mask, torch.uint8)
        self.grid = make_grid(self.z.shape[0], self.z.shape[1], cell_size, boundary_conditions)
        self.options = LemOptions(timestep, erodibility, m_exponent, n_exponent, uplift_rate, hillslope_diffusivity,
                                  slope_clamp, baselevel_fall_rate, fill_min_slope, int(enable_hillslope),
                                  int(divide_area_by_dx), hillslope_rel_tol, hillslope_max_iter,
                                  int(hillslope_nonlinear), critical_slope)
        h = ctypes.c_void_p()
        _check(L.lsdtt_gpu_lem_create(ctypes.byref(self.grid), ctypes.c_void_p(self.mask.data_ptr()),
                                      ctypes.byref(self.options), ctypes.byref(h), _stream(stream)))
        self._h = h

    def set_preconditioner(self, net: Optional["UNet"]):
        """Use a trained UNet in the hillslope solves (None: Jacobi-PCG)."""
        fn = lib().lsdtt_gpu_lem_set_preconditioner
        fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        fn.restype = ctypes.c_int
        _check(fn(self._h, net._h if net is not None else None))
        self._net = net  # keep it alive while attached

    def step(self, stream=None, want_stats=True):
        st = LemStats()
        _check(lib().lsdtt_gpu_lem_step(self._h, ctypes.c_void_p(self.z.data_ptr()),
                                        ctypes.byref(st) if want_stats else None, _stream(stream)))
        return st.as_dict() if want_stats else None

    def close(self):
        if getattr(self, "_h", None):
            lib().lsdtt_gpu_lem_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Ensemble:
    """A batched ensemble of independent LEM runs (lsdtt_gpu_ensemble_*):
    every member advances exactly as LandscapeModel.step would advance it
    alone, all members in one launch per stage, one CUDA graph per step.

    members: sequence of dicts with z, mask (optional), cell_size,
    boundary_conditions and any LandscapeModel option."""

    _DEFAULTS = dict(timestep=100.0, erodibility=1e-3, m_exponent=0.45, n_exponent=1.0, uplift_rate=1e-4,
                     hillslope_diffusivity=1e-3, slope_clamp=1e-5, baselevel_fall_rate=0.0, fill_min_slope=0.0,
                     enable_hillslope=True, divide_area_by_dx=True, hillslope_rel_tol=1e-8, hillslope_max_iter=2000)

    def __init__(self, members, use_graph=True, stream=None):
        torch = _torch()
        L = _bind_more()
        arr = (Member * len(members))()
        self.shapes = []
        for k, spec in enumerate(members):
            spec = dict(spec)
            z = np.asarray(spec.pop("z"), np.float32)
            spec.pop("mask", None)
            cell = spec.pop("cell_size")
            bc = spec.pop("boundary_conditions", "oooo")
            o = dict(self._DEFAULTS)
            unknown = set(spec) - set(o)
            if unknown:
                raise TypeError(f"unknown member options {sorted(unknown)}")
            o.update(spec)
            arr[k].grid = make_grid(z.shape[0], z.shape[1], cell, bc)
            arr[k].options = LemOptions(o["timestep"], o["erodibility"], o["m_exponent"], o["n_exponent"],
                                        o["uplift_rate"], o["hillslope_diffusivity"], o["slope_clamp"],
                                        o["baselevel_fall_rate"], o["fill_min_slope"], int(o["enable_hillslope"]),
                                        int(o["divide_area_by_dx"]), o["hillslope_rel_tol"], o["hillslope_max_iter"],
                                        0, 1.0)
            self.shapes.append(z.shape)
        h = ctypes.c_void_p()
        _check(L.lsdtt_gpu_ensemble_create(arr, len(members), int(use_graph), ctypes.byref(h), _stream(stream)))
        self._h = h
        self.n_members = len(members)
        for k, spec in enumerate(members):
            zt = _dev(spec["z"], torch.float32)
            m = spec.get("mask")
            mt = _dev(np.ones(zt.shape, np.uint8) if m is None else m, torch.uint8)
            _check(L.lsdtt_gpu_ensemble_set_member(self._h, k, ctypes.c_void_p(zt.data_ptr()),
                                                   ctypes.c_void_p(mt.data_ptr()), _stream(stream)))

    def step(self, n_steps=1, want_stats=False, stream=None):
        stats = (LemStats * self.n_members)() if want_stats else None
        _check(lib().lsdtt_gpu_ensemble_step(self._h, n_steps, stats, _stream(stream)))
        return [s.as_dict() for s in stats] if want_stats else None

    def set(self, k, z, mask=None, stream=None):
        """Replace member k's surface between steps. With a mask, the mask
        too (which also fixes its boundary flats; the next step captures its
        graph again); without one, only the elevations (the captured step
        stays)."""
        torch = _torch()
        zt = _dev(z, torch.float32)
        if tuple(zt.shape) != tuple(self.shapes[k]):
            raise ValueError(f"member {k} is {self.shapes[k]}, got {tuple(zt.shape)}")
        if mask is None:
            _check(lib().lsdtt_gpu_ensemble_set_surface(self._h, k, ctypes.c_void_p(zt.data_ptr()), _stream(stream)))
        else:
            mt = _dev(mask, torch.uint8)
            _check(lib().lsdtt_gpu_ensemble_set_member(self._h, k, ctypes.c_void_p(zt.data_ptr()),
                                                       ctypes.c_void_p(mt.data_ptr()), _stream(stream)))
        (stream or torch.cuda.current_stream()).synchronize()

    def get(self, k, stream=None):
        torch = _torch()
        out = torch.empty(self.shapes[k], dtype=torch.float32, device="cuda")
        _check(lib().lsdtt_gpu_ensemble_get_member(self._h, k, ctypes.c_void_p(out.data_ptr()), _stream(stream)))
        return out

    def offsets(self):
        off = np.empty(self.n_members + 1, np.int64)
        _check(lib().lsdtt_gpu_ensemble_offsets(self._h, off.ctypes.data))
        return off

    def override_schedule(self, fill_pass_cap=0, hillslope_iteration_cap=0, sweep_mode=-1):
        """Force a schedule (tests): caps for the next capture; sweep_mode 0
        (level launches), 1 (dataflow), 2 (cooperative levels), 3 (member
        clusters) or -1 (autotuned)."""
        _check(lib().lsdtt_gpu_ensemble_override_schedule(self._h, fill_pass_cap, hillslope_iteration_cap,
                                                          sweep_mode))

    def set_member_groups(self, enabled: bool) -> None:
        """Member groups of captured steps (the deep members' sweep beside
        the others' sweep and hillslope solve); off by default, same results."""
        _check(lib().lsdtt_gpu_ensemble_set_member_groups(self._h, 1 if enabled else 0))

    def info(self):
        i = EnsembleInfo()
        _check(lib().lsdtt_gpu_ensemble_get_info(self._h, ctypes.byref(i)))
        return i.as_dict()

    def close(self):
        if getattr(self, "_h", None):
            lib().lsdtt_gpu_ensemble_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DinfView(ctypes.Structure):
    _fields_ = [("receivers", ctypes.c_void_p), ("weights", ctypes.c_void_p), ("n_receivers", ctypes.c_void_p),
                ("slope", ctypes.c_void_p), ("bearing", ctypes.c_void_p), ("donor_count", ctypes.c_void_p),
                ("topological_order", ctypes.c_void_p), ("n_cells", ctypes.c_int64), ("n_valid_cells", ctypes.c_int64),
                ("n_levels", ctypes.c_int64)]


class FlowGraphDinf:
    """The D-infinity flow graph (lsdtt_flowgraph_cpu with method
    d_infinity) on the GPU: receivers and weights, facet slopes and
    bearings, donor counts, the topological order, accumulate() and
    D-infinity stream power. Accessors return CUDA tensors valid until the
    next build() or close()."""

    def __init__(self, z, mask, cell_size, boundary_conditions="oooo", *, interior_nodata_is_outlet=True,
                 no_data_value=-9999.0, stream=None):
        torch = _torch()
        L = lib()
        vp = ctypes.c_void_p
        for name, args in {"lsdtt_gpu_dinf_create": [ctypes.POINTER(Grid), ctypes.POINTER(vp)],
                           "lsdtt_gpu_dinf_destroy": [vp],
                           "lsdtt_gpu_dinf_build": [vp, vp, vp, ctypes.c_int32, vp],
                           "lsdtt_gpu_dinf_get_view": [vp, ctypes.POINTER(DinfView)],
                           "lsdtt_gpu_dinf_accumulate": [vp, vp, vp, vp],
                           "lsdtt_gpu_dinf_stream_power": [vp, vp, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                                           ctypes.c_float, ctypes.c_float, ctypes.c_int32,
                                                           ctypes.c_float, vp, vp]}.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        zt = _dev(z, torch.float32)
        self.shape = tuple(zt.shape)
        self.grid = make_grid(zt.shape[0], zt.shape[1], cell_size, boundary_conditions, no_data_value)
        h = vp()
        _check(L.lsdtt_gpu_dinf_create(ctypes.byref(self.grid), ctypes.byref(h)))
        self._h = h
        self._inio = int(bool(interior_nodata_is_outlet))
        self.build(zt, mask, stream=stream)

    def build(self, z, mask, stream=None):
        torch = _torch()
        self._z = _dev(z, torch.float32)
        self._m = _dev(mask, torch.uint8)
        _check(lib().lsdtt_gpu_dinf_build(self._h, ctypes.c_void_p(self._z.data_ptr()),
                                          ctypes.c_void_p(self._m.data_ptr()), self._inio, _stream(stream)))
        v = DinfView()
        _check(lib().lsdtt_gpu_dinf_get_view(self._h, ctypes.byref(v)))
        self.view = v

    def _arr(self, ptr, count, dtype, shape=None):
        """Zero-copy CUDA tensor over a graph-owned device array."""
        torch = _torch()
        if not ptr or not count:
            return torch.empty(0 if shape is None else shape, dtype=dtype, device="cuda")
        t = torch.as_tensor(_DeviceArray(ptr, int(count), dtype), device="cuda")
        return t if shape is None else t.reshape(shape)

    def receivers(self):
        torch = _torch()
        return self._arr(self.view.receivers, 2 * self.view.n_cells, torch.int64, (self.view.n_cells, 2))

    def weights(self):
        torch = _torch()
        return self._arr(self.view.weights, 2 * self.view.n_cells, torch.float32, (self.view.n_cells, 2))

    def n_receivers(self):
        torch = _torch()
        return self._arr(self.view.n_receivers, self.view.n_cells, torch.uint8)

    def slopes(self):
        torch = _torch()
        return self._arr(self.view.slope, self.view.n_cells, torch.float32)

    def bearings(self):
        torch = _torch()
        return self._arr(self.view.bearing, self.view.n_cells, torch.float32)

    def donor_count(self):
        torch = _torch()
        return self._arr(self.view.donor_count, self.view.n_cells, torch.uint8)

    def topological_order(self):
        torch = _torch()
        return self._arr(self.view.topological_order, self.view.n_valid_cells, torch.int64)

    def accumulate(self, weights=None, stream=None):
        torch = _torch()
        out = torch.empty(self.view.n_cells, dtype=torch.float64, device="cuda")
        w = None if weights is None else _dev(weights, torch.float64).reshape(-1)
        _check(lib().lsdtt_gpu_dinf_accumulate(self._h, ctypes.c_void_p(w.data_ptr() if w is not None else 0),
                                               ctypes.c_void_p(out.data_ptr()), _stream(stream)))
        return out

    def stream_power(self, K, m, n, dt, incision_threshold_area=0.0, divide_area_by_dx=True, slope_clamp=1e-5,
                     stream=None):
        """compute_dinf_stream_power_incision on the surface the graph was built on."""
        torch = _torch()
        out = torch.empty_like(self._z)
        _check(lib().lsdtt_gpu_dinf_stream_power(self._h, ctypes.c_void_p(self._z.data_ptr()), K, m, n, dt,
                                                 incision_threshold_area, int(bool(divide_area_by_dx)), slope_clamp,
                                                 ctypes.c_void_p(out.data_ptr()), _stream(stream)))
        return out

    def close(self):
        if getattr(self, "_h", None):
            lib().lsdtt_gpu_dinf_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def hillslope_implicit(z, mask, cell_size, boundary_conditions, D, Sc, dt, nonlinear=True, rel_tol=1e-8,
                       max_pcg_iter=4000, residual_tol=1e-12, max_outer=200, is_channel=None, net=None, stream=None):
    """Backward-Euler hillslope step over dt (linear or Roering), the
    reference's compute_hillslope_newton_transient. With `net` (a UNet) the
    linear systems are solved by flexible PCG with the network as the
    preconditioner, checked and finished by Jacobi-PCG. Returns (z CUDA
    tensor, SolveReport with the total PCG iteration count)."""
    torch = _torch()
    L = _bind_more()
    vp = ctypes.c_void_p
    args = [ctypes.POINTER(Grid), vp, vp, vp, ctypes.c_float, ctypes.c_float, ctypes.c_int32, ctypes.c_float,
            ctypes.c_double, ctypes.c_int32, ctypes.c_double, ctypes.c_int32]
    if net is None:
        fn = L.lsdtt_gpu_hillslope_implicit
        fn.argtypes = args + [vp, ctypes.POINTER(SolveReport), vp]
    else:
        fn = L.lsdtt_gpu_hillslope_implicit_learned
        fn.argtypes = args + [vp, vp, ctypes.POINTER(SolveReport), vp]
    fn.restype = ctypes.c_int
    zt = _dev(z, torch.float32)
    mt = _dev(mask, torch.uint8)
    ct = None if is_channel is None else _dev(is_channel, torch.uint8)
    g = make_grid(zt.shape[0], zt.shape[1], cell_size, boundary_conditions)
    out = torch.empty_like(zt)
    rep = SolveReport()
    head = [ctypes.byref(g), vp(zt.data_ptr()), vp(mt.data_ptr()), vp(ct.data_ptr() if ct is not None else 0),
            ctypes.c_float(D), ctypes.c_float(Sc), ctypes.c_int32(int(nonlinear)), ctypes.c_float(dt),
            ctypes.c_double(rel_tol), ctypes.c_int32(max_pcg_iter), ctypes.c_double(residual_tol),
            ctypes.c_int32(max_outer)]
    tail = [vp(out.data_ptr()), ctypes.byref(rep), _stream(stream)]
    _check(fn(*head, *tail) if net is None else fn(*head, net._h, *tail))
    return out, rep


# U-Net layer table: (name, Cin, Cout), the order of the parameter vector
# (weights [Cout][3][3][Cin] of every layer, then every bias).
UNET_LAYERS = [("enc0", 1, 16), ("enc1", 16, 32), ("enc2", 32, 64), ("enc3", 64, 64), ("dec2", 64, 64),
               ("dec1", 64, 32), ("dec0", 32, 16), ("out", 16, 1)]


def unet_flatten(params: dict) -> np.ndarray:
    """{name.w, name.b} -> the library's flat FP32 parameter vector."""
    parts = [np.asarray(params[n + ".w"], np.float32).reshape(-1) for n, _, _ in UNET_LAYERS]
    parts += [np.asarray(params[n + ".b"], np.float32).reshape(-1) for n, _, _ in UNET_LAYERS]
    return np.concatenate(parts)


def unet_unflatten(vec) -> dict:
    vec = np.asarray(vec, np.float32)
    out, o = {}, 0
    for n, ci, co in UNET_LAYERS:
        k = co * 9 * ci
        out[n + ".w"] = vec[o:o + k].reshape(co, 3, 3, ci)
        o += k
    for n, ci, co in UNET_LAYERS:
        out[n + ".b"] = vec[o:o + co].copy()
        o += co
    return out


class UNet:
    """The learned hillslope preconditioner (lsdtt_gpu_unet_*): forward,
    gradient and optimiser steps all run in liblsdtt_gb300.so."""

    def __init__(self, max_rows: int, max_cols: int, seed: int = 1):
        L = lib()
        vp, i32, i64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
        for name, args, res in [
            ("lsdtt_gpu_unet_create", [i32, i32, ctypes.c_uint64, ctypes.POINTER(vp)], ctypes.c_int),
            ("lsdtt_gpu_unet_destroy", [vp], ctypes.c_int),
            ("lsdtt_gpu_unet_num_params", [vp], i64),
            ("lsdtt_gpu_unet_get_params", [vp, vp, i64], ctypes.c_int),
            ("lsdtt_gpu_unet_set_params", [vp, vp, i64], ctypes.c_int),
            ("lsdtt_gpu_unet_apply", [vp, vp, i32, i32, vp, vp], ctypes.c_int),
            ("lsdtt_gpu_unet_loss_grad", [vp, vp, vp, i32, i32, ctypes.POINTER(ctypes.c_double), vp, vp],
             ctypes.c_int),
            ("lsdtt_gpu_unet_train_step", [vp, vp, vp, i32, i32, i32, ctypes.c_float,
                                           ctypes.POINTER(ctypes.c_double), vp], ctypes.c_int),
            ("lsdtt_gpu_unet_set_conv_kernel", [vp, i32], ctypes.c_int),
            ("lsdtt_gpu_unet_status", [vp], ctypes.c_int),
        ]:
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        h = vp()
        _check(L.lsdtt_gpu_unet_create(max_rows, max_cols, seed, ctypes.byref(h)))
        self._h = h
        self.n_params = int(L.lsdtt_gpu_unet_num_params(h))

    def set_conv_kernel(self, kind: str) -> None:
        """'mma' (mma.sync m16n8k16), 'tcgen05' (UMMA, accumulator in TMEM),
        'tcgen05_rows' (UMMA over rolling input rows) or 'tcgen05_ws' (the
        rolling-row form with warp-specialised producer, MMA and epilogue
        roles; the default)."""
        _check(lib().lsdtt_gpu_unet_set_conv_kernel(self._h, {"mma": 0, "tcgen05": 1, "tcgen05_rows": 2, "tcgen05_ws": 3}[kind]))

    def status(self) -> None:
        """Raises if a tensor-core convolution gave up waiting for its MMAs."""
        _check(lib().lsdtt_gpu_unet_status(self._h))

    def get_params(self) -> np.ndarray:
        out = np.empty(self.n_params, np.float32)
        _check(lib().lsdtt_gpu_unet_get_params(self._h, out.ctypes.data, self.n_params))
        return out

    def set_params(self, vec) -> None:
        vec = np.ascontiguousarray(vec, np.float32)
        if vec.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters, got {vec.size}")
        _check(lib().lsdtt_gpu_unet_set_params(self._h, vec.ctypes.data, self.n_params))

    def apply(self, r, stream=None):
        torch = _torch()
        rt = _dev(r, torch.float32)
        y = torch.empty_like(rt)
        _check(lib().lsdtt_gpu_unet_apply(self._h, ctypes.c_void_p(rt.data_ptr()), rt.shape[0], rt.shape[1],
                                          ctypes.c_void_p(y.data_ptr()), _stream(stream)))
        return y

    def loss_grad(self, r, e, stream=None):
        torch = _torch()
        rt, et = _dev(r, torch.float32), _dev(e, torch.float32)
        loss = ctypes.c_double()
        g = np.empty(self.n_params, np.float32)
        _check(lib().lsdtt_gpu_unet_loss_grad(self._h, ctypes.c_void_p(rt.data_ptr()), ctypes.c_void_p(et.data_ptr()),
                                              rt.shape[0], rt.shape[1], ctypes.byref(loss), g.ctypes.data,
                                              _stream(stream)))
        return loss.value, g

    def train_step(self, r, e, lr=1e-3, optimizer="adam", stream=None) -> float:
        torch = _torch()
        rt, et = _dev(r, torch.float32), _dev(e, torch.float32)
        loss = ctypes.c_double()
        _check(lib().lsdtt_gpu_unet_train_step(self._h, ctypes.c_void_p(rt.data_ptr()),
                                               ctypes.c_void_p(et.data_ptr()), rt.shape[0], rt.shape[1],
                                               {"sgd": 0, "adam": 1}[optimizer], ctypes.c_float(lr),
                                               ctypes.byref(loss), _stream(stream)))
        return loss.value

    def close(self):
        if getattr(self, "_h", None):
            lib().lsdtt_gpu_unet_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def capture_pairs(z, mask, cell_size, boundary_conditions, D, Sc, dt, n_pairs, nonlinear=True, rel_tol=1e-8,
                  max_iter=4000, is_channel=None, stream=None):
    """Residual/correction pairs from the plain Jacobi-PCG solve
    (lsdtt_gpu_hillslope_capture_pairs). Returns (r, e) CUDA tensors of shape
    [k, n_rows, n_cols], r scaled to metres (dt * residual)."""
    torch = _torch()
    L = lib()
    vp = ctypes.c_void_p
    fn = L.lsdtt_gpu_hillslope_capture_pairs
    fn.argtypes = [ctypes.POINTER(Grid), vp, vp, vp, ctypes.c_float, ctypes.c_float, ctypes.c_int32, ctypes.c_float,
                   ctypes.c_double, ctypes.c_int32, ctypes.c_int32, vp, vp, ctypes.POINTER(ctypes.c_int32), vp]
    fn.restype = ctypes.c_int
    zt = _dev(z, torch.float32)
    mt = _dev(mask, torch.uint8)
    ct = None if is_channel is None else _dev(is_channel, torch.uint8)
    g = make_grid(zt.shape[0], zt.shape[1], cell_size, boundary_conditions)
    r = torch.empty((n_pairs,) + tuple(zt.shape), dtype=torch.float32, device=zt.device)
    e = torch.empty_like(r)
    k = ctypes.c_int32()
    _check(fn(ctypes.byref(g), vp(zt.data_ptr()), vp(mt.data_ptr()), vp(ct.data_ptr() if ct is not None else 0),
              ctypes.c_float(D), ctypes.c_float(Sc), ctypes.c_int32(int(nonlinear)), ctypes.c_float(dt),
              ctypes.c_double(rel_tol), ctypes.c_int32(max_iter), ctypes.c_int32(n_pairs), vp(r.data_ptr()),
              vp(e.data_ptr()), ctypes.byref(k), _stream(stream)))
    return r[:k.value], e[:k.value]
