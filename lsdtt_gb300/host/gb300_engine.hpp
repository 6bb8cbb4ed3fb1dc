// gb300_engine.hpp -- the C++ host layer of the GB300 backend, over the C ABI
// of include/lsdtt_gb300.h, with no dependency on lsdtt3's own headers.
//
// It holds what a C++ caller of the hot path needs: the D8 engine with host
// mirrors of every component and the queries of lsdtt_flow_base
// (src/core/lsdtt_flow_base.hpp:126-491), the epsilon fill
// (fill_pits, src/cpu/lsdtt_raster_flow_preprocessing_cpu.hpp:191-199), D8
// stream power (compute_d8_stream_power_incision,
// src/cpu/lsdtt_stream_power_cpu.hpp:74-89) and the LEM timestep
// (run_lem_step, src/cpu/lsdtt_lem_cpu.hpp:223-232), on host arrays.
// lsdtt_flowinfo_gpu.hpp and lsdtt_gpu_overloads.hpp wrap it in the
// reference's own types; this layer compiles and runs without them.
//
// Errors are thrown as the reference throws them: std::invalid_argument for
// a bad forced outlet, std::runtime_error with the reference's message
// otherwise (the message of lsdtt_gpu_last_error()). gb300_error carries the
// C status as well. Device memory is owned by RAII buffers; every call is
// synchronous on the legacy default stream.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "lsdtt_gb300.h"

namespace lsdtt_gb300_host
{

class gb300_error : public std::runtime_error
{
public:
    gb300_error(int status, const std::string& msg) : std::runtime_error(msg), status_(status) {}
    int status() const noexcept { return status_; }

private:
    int status_;
};

inline void check(int st)
{
    if (st == LSDTT_GPU_OK) return;
    const std::string msg = lsdtt_gpu_last_error();
    if (st == LSDTT_GPU_EINVAL && msg.find("forced outlet") != std::string::npos) throw std::invalid_argument(msg);
    throw gb300_error(st, msg);
}

inline void check_cuda(cudaError_t e, const char* where)
{
    if (e != cudaSuccess) throw gb300_error(LSDTT_GPU_ECUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// A device array of n elements; copied in from / out to host vectors.
template <class T>
class device_buffer
{
public:
    device_buffer() = default;
    explicit device_buffer(std::size_t n) : n_(n)
    {
        if (n) check_cuda(cudaMalloc(&p_, sizeof(T) * n), "device_buffer");
    }
    device_buffer(const T* host, std::size_t n) : device_buffer(n)
    {
        if (n) check_cuda(cudaMemcpy(p_, host, sizeof(T) * n, cudaMemcpyHostToDevice), "device_buffer upload");
    }
    ~device_buffer() { if (p_) cudaFree(p_); }
    device_buffer(const device_buffer&) = delete;
    device_buffer& operator=(const device_buffer&) = delete;
    device_buffer(device_buffer&& o) noexcept : p_(o.p_), n_(o.n_) { o.p_ = nullptr; o.n_ = 0; }
    device_buffer& operator=(device_buffer&& o) noexcept
    {
        std::swap(p_, o.p_);
        std::swap(n_, o.n_);
        return *this;
    }
    T* get() const noexcept { return p_; }
    std::size_t size() const noexcept { return n_; }
    std::vector<T> to_host() const
    {
        std::vector<T> out(n_);
        if (n_) check_cuda(cudaMemcpy(out.data(), p_, sizeof(T) * n_, cudaMemcpyDeviceToHost), "device_buffer download");
        return out;
    }
    void from_host(const T* host)
    {
        if (n_) check_cuda(cudaMemcpy(p_, host, sizeof(T) * n_, cudaMemcpyHostToDevice), "device_buffer upload");
    }

private:
    T* p_ = nullptr;
    std::size_t n_ = 0;
};

// lsdtt_raster_meta reduced to what the path reads, plus the NESW boundary
// string (lsdtt_flowinfo_options::boundary_conditions).
struct grid
{
    int n_rows = 0;
    int n_cols = 0;
    double cell_size = 1.0;
    double no_data_value = -9999.0;
    std::string boundary_conditions = "oooo";

    std::size_t cells() const noexcept { return static_cast<std::size_t>(n_rows) * static_cast<std::size_t>(n_cols); }
    lsdtt_gpu_grid c_grid() const
    {
        if (boundary_conditions.size() != 4)
            throw std::runtime_error(
                "lsdtt_flowinfo: boundary_conditions must have length 4 (north, east, south, west)");
        lsdtt_gpu_grid g{};
        g.n_rows = n_rows;
        g.n_cols = n_cols;
        g.cell_size = cell_size;
        g.no_data_value = no_data_value;
        std::memcpy(g.boundary_conditions, boundary_conditions.data(), 4);
        return g;
    }
};

// lsdtt_flowinfo_options (src/core/lsdtt_flow_base.hpp:79-111).
struct flow_options
{
    bool interior_nodata_is_outlet = true;
    bool require_acyclic_graph = true;
    bool build_topological_order = true;
    bool build_s_vector = true;
    bool allow_pits_as_outlets = false;
    std::vector<std::int64_t> forced_outlet_flats;
};

// fill_pits(raster, min_slope, bc): returns the filled elevations (masked and
// nodata cells hold the no-data value).
inline std::vector<float> fill_pits(const grid& g, const float* z, const std::uint8_t* mask, float min_slope)
{
    const lsdtt_gpu_grid cg = g.c_grid();
    device_buffer<float> zd(z, g.cells()), out(g.cells());
    device_buffer<std::uint8_t> md(mask, g.cells());
    check(lsdtt_gpu_fill_pits(&cg, zd.get(), md.get(), min_slope, out.get(), nullptr));
    return out.to_host();
}

// The D8 engine: builds every component on the GPU, then mirrors them to host
// memory once, so every const query is a host read (safe to call
// concurrently; upslope slices stay valid for the engine's lifetime,
// flow_base.hpp:56-57, 198-204).
class flow_engine
{
public:
    flow_engine(const grid& g, const float* z, const std::uint8_t* mask, const flow_options& o = flow_options{})
        : grid_(g), mask_(mask, mask + g.cells())
    {
        const lsdtt_gpu_grid cg = g.c_grid();
        check(lsdtt_gpu_flow_create(&cg, &flow_));
        try
        {
            const std::size_t n = g.cells();
            zd_ = device_buffer<float>(z, n);
            md_ = device_buffer<std::uint8_t>(mask, n);
            device_buffer<std::int64_t> fd(o.forced_outlet_flats.data(), o.forced_outlet_flats.size());
            const lsdtt_gpu_flow_options co{o.interior_nodata_is_outlet ? 1 : 0, o.require_acyclic_graph ? 1 : 0,
                                            o.build_topological_order ? 1 : 0, o.build_s_vector ? 1 : 0,
                                            o.allow_pits_as_outlets ? 1 : 0};
            check(lsdtt_gpu_flow_build(flow_, zd_.get(), md_.get(), &co, fd.get(),
                                       static_cast<std::int64_t>(o.forced_outlet_flats.size()), nullptr));
            lsdtt_gpu_flow_view v{};
            check(lsdtt_gpu_flow_get_view(flow_, &v));
            pull(receiver_, v.receiver, n);
            pull(dir_, v.direction, n);
            pull(donors_, v.donor_count, n);
            pull(outlets_, v.outlets, static_cast<std::size_t>(v.n_outlets));
            if (v.has_topological_order) pull(topo_, v.topological_order, static_cast<std::size_t>(v.n_valid_cells));
            if (v.has_s_vector)
            {
                pull(svec_, v.s_vector, static_cast<std::size_t>(v.n_valid_cells));
                pull(start_, v.s_vector_start, n);
                pull(size_, v.s_vector_size, n);
            }
            n_valid_ = v.n_valid_cells;
            acyclic_ = v.is_acyclic != 0;
            has_topo_ = v.has_topological_order != 0;
            has_sv_ = v.has_s_vector != 0;
        }
        catch (...)
        {
            lsdtt_gpu_flow_destroy(flow_);
            throw;
        }
    }
    ~flow_engine() { lsdtt_gpu_flow_destroy(flow_); }
    flow_engine(const flow_engine&) = delete;
    flow_engine& operator=(const flow_engine&) = delete;

    // ---- state -------------------------------------------------------------
    const grid& geometry() const noexcept { return grid_; }
    bool empty() const noexcept { return n_valid_ == 0; }
    bool is_acyclic() const noexcept { return acyclic_; }
    bool has_s_vector() const noexcept { return has_sv_; }
    bool has_topological_order() const noexcept { return has_topo_; }
    std::int64_t n_valid_cells() const noexcept { return n_valid_; }
    std::size_t full_grid_size() const noexcept { return mask_.size(); }

    // ---- indexing ----------------------------------------------------------
    bool in_bounds(int r, int c) const noexcept { return r >= 0 && r < grid_.n_rows && c >= 0 && c < grid_.n_cols; }
    bool is_flat_in_range(std::int64_t f) const noexcept
    {
        return f >= 0 && f < static_cast<std::int64_t>(mask_.size());
    }
    std::int64_t flat_index_unchecked(int r, int c) const noexcept
    {
        return static_cast<std::int64_t>(r) * grid_.n_cols + c;
    }
    std::int64_t flat_index(int r, int c) const
    {
        if (!in_bounds(r, c)) throw std::out_of_range("lsdtt_flowinfo: row/col out of range");
        return flat_index_unchecked(r, c);
    }
    int row_from_flat(std::int64_t f) const { require_range(f); return static_cast<int>(f / grid_.n_cols); }
    int col_from_flat(std::int64_t f) const { require_range(f); return static_cast<int>(f % grid_.n_cols); }
    bool is_valid_cell(std::int64_t f) const noexcept { return is_flat_in_range(f) && mask_[f] != 0; }

    // ---- receivers, donors, outlets ------------------------------------------
    const std::vector<std::int64_t>& receivers() const noexcept { return receiver_; }
    const std::vector<std::uint8_t>& directions() const noexcept { return dir_; }
    const std::vector<std::uint8_t>& donor_counts() const noexcept { return donors_; }
    const std::vector<std::int64_t>& outlets() const noexcept { return outlets_; }
    const std::vector<std::int64_t>& topological_order() const
    {
        if (!has_topo_) throw std::runtime_error("lsdtt_flowinfo: topological_order was not built for this object");
        return topo_;
    }
    const std::vector<std::int64_t>& s_vector() const { need_sv(); return svec_; }
    const std::vector<std::int64_t>& s_vector_starts() const { need_sv(); return start_; }
    const std::vector<std::uint64_t>& s_vector_sizes() const { need_sv(); return size_; }

    bool is_outlet(std::int64_t f) const { require_valid(f); return receiver_[f] == -2; }
    std::int64_t receiver_of(std::int64_t f) const { require_valid(f); return receiver_[f]; }
    std::uint8_t receiver_dir_of(std::int64_t f) const { require_valid(f); return dir_[f]; }
    std::uint8_t donor_count_of(std::int64_t f) const { require_valid(f); return donors_[f]; }

    // ---- s-vector ------------------------------------------------------------
    std::int64_t s_vector_start(std::int64_t f) const { require_sv(f); return start_[f]; }
    std::uint64_t s_vector_size(std::int64_t f) const { require_sv(f); return size_[f]; }
    // The cells upslope of f, f first, in the reference's s-vector order.
    std::pair<const std::int64_t*, std::size_t> upslope_nodes(std::int64_t f) const
    {
        require_sv(f);
        return {svec_.data() + start_[f], static_cast<std::size_t>(size_[f])};
    }
    bool is_upslope_of(std::int64_t cand, std::int64_t target) const
    {
        require_sv(cand);
        require_sv(target);
        const std::int64_t a = start_[target], s = start_[cand];
        return s >= a && s < a + static_cast<std::int64_t>(size_[target]);
    }

    // lsdtt_flowinfo::accumulate (flowinfo_cpu.cpp:1979-2046) on the GPU: the
    // seed is dx^2 per valid cell, or the given per-cell weights.
    std::vector<double> accumulate(const std::vector<double>& weights = {}) const
    {
        const std::size_t n = mask_.size();
        if (!weights.empty() && weights.size() != n)
            throw std::invalid_argument("lsdtt_flowinfo::accumulate: cell_weights size must equal n_rows * n_cols");
        device_buffer<double> wd(weights.data(), weights.size()), od(n);
        check(lsdtt_gpu_flow_accumulate(flow_, weights.empty() ? nullptr : wd.get(), od.get(), nullptr));
        return od.to_host();
    }

    // The query rasters of lsdtt_flow_base (flowinfo_cpu.cpp:2255-2965):
    // kind as lsdtt_gpu_flow_query; values / value_mask / channel_mask are
    // the reference method's elev (or values), elev_mask (valid_mask) and
    // channel_mask (sink_mask) where it takes them.
    struct raster_out
    {
        std::vector<float> data;
        std::vector<std::uint8_t> mask;
        std::vector<std::int64_t> donor;  // kind 2 only
    };
    raster_out query(int kind, const std::vector<float>& values = {}, const std::vector<std::uint8_t>& value_mask = {},
                     const std::vector<std::uint8_t>& channel_mask = {}, int threshold = 1,
                     bool include_self = true) const
    {
        const std::size_t n = mask_.size();
        auto sized = [&](std::size_t k) { return k == 0 || k == n; };
        if (!sized(values.size()) || !sized(value_mask.size()) || !sized(channel_mask.size()))
            throw std::invalid_argument(
                "lsdtt_flowinfo: query inputs must have the same flat-index size as the DEM");
        device_buffer<float> vd(values.data(), values.size()), od(n);
        device_buffer<std::uint8_t> vm(value_mask.data(), value_mask.size()), cm(channel_mask.data(),
                                                                                   channel_mask.size()),
            om(n);
        device_buffer<std::int64_t> dd(kind == 2 ? n : 0);
        check(lsdtt_gpu_flow_query(flow_, kind, values.empty() ? nullptr : vd.get(),
                                   value_mask.empty() ? nullptr : vm.get(), channel_mask.empty() ? nullptr : cm.get(),
                                   threshold, include_self ? 1 : 0, od.get(), om.get(), kind == 2 ? dd.get() : nullptr,
                                   nullptr));
        raster_out r;
        r.data = od.to_host();
        r.mask = om.to_host();
        if (kind == 2) r.donor = dd.to_host();
        return r;
    }

    // The engine's C handle and its device copies of the DEM and the mask
    // (for the stream-power call, which reads the routing on the device).
    lsdtt_gpu_flow* handle() const noexcept { return flow_; }
    const float* dem_device() const noexcept { return zd_.get(); }

private:
    template <class T>
    static void pull(std::vector<T>& dst, const T* src, std::size_t n)
    {
        dst.resize(n);
        if (n) check_cuda(cudaMemcpy(dst.data(), src, sizeof(T) * n, cudaMemcpyDeviceToHost), "flow_engine");
    }
    void require_range(std::int64_t f) const
    {
        if (!is_flat_in_range(f)) throw std::out_of_range("lsdtt_flowinfo: flat index out of range");
    }
    void require_valid(std::int64_t f) const
    {
        require_range(f);
        if (!mask_[f]) throw std::invalid_argument("lsdtt_flowinfo: cell is not a valid cell");
    }
    void need_sv() const
    {
        if (!has_sv_)
            throw std::runtime_error(
                "lsdtt_flowinfo: s_vector not built - set build_s_vector = true in lsdtt_flowinfo_options");
    }
    void require_sv(std::int64_t f) const
    {
        require_valid(f);
        if (!has_sv_) throw std::runtime_error("lsdtt_flowinfo: s_vector was not built for this object");
    }

    grid grid_;
    lsdtt_gpu_flow* flow_ = nullptr;
    device_buffer<float> zd_;
    device_buffer<std::uint8_t> md_;
    std::vector<std::uint8_t> mask_;
    std::vector<std::int64_t> receiver_, outlets_, topo_, svec_, start_;
    std::vector<std::uint8_t> dir_, donors_;
    std::vector<std::uint64_t> size_;
    std::int64_t n_valid_ = 0;
    bool acyclic_ = false, has_topo_ = false, has_sv_ = false;
};

// compute_d8_stream_power_incision on the engine's routing: one implicit
// stream-power step of z (the surface the engine was built on, or any
// surface of the same grid) over dt. erodibility_field: empty, or one K per
// cell.
inline std::vector<float> stream_power_d8(const flow_engine& flow, const float* z, float K, float m, float n, float dt,
                                          float incision_threshold_area = 0.0f, bool divide_area_by_dx = true,
                                          float slope_clamp = 1e-5f,
                                          const std::vector<float>& erodibility_field = {})
{
    const std::size_t cells = flow.full_grid_size();
    if (!erodibility_field.empty() && erodibility_field.size() != cells)
        throw std::invalid_argument(
            "compute_d8_stream_power_incision: erodibility_field must be empty or hold n_rows*n_cols values");
    device_buffer<float> zd(z, cells), out(cells), kd(erodibility_field.data(), erodibility_field.size());
    check(lsdtt_gpu_stream_power_d8(flow.handle(), zd.get(), erodibility_field.empty() ? nullptr : kd.get(), K, m, n,
                                    dt, incision_threshold_area, divide_area_by_dx ? 1 : 0, slope_clamp, out.get(),
                                    nullptr));
    return out.to_host();
}

// run_lem_step in the D8 coupled regime with the implicit hillslope
// (linear, or the Roering law), optionally preceded by the epsilon fill.
// The engine keeps its buffers across steps; boundary flats come from the
// mask and the boundary string (build_boundary_flats, lem_cpu.cpp:735-808).
class lem_engine
{
public:
    lem_engine(const grid& g, const std::uint8_t* mask, const lsdtt_gpu_lem_options& o) : grid_(g), zd_(g.cells())
    {
        const lsdtt_gpu_grid cg = g.c_grid();
        device_buffer<std::uint8_t> md(mask, g.cells());
        check(lsdtt_gpu_lem_create(&cg, md.get(), &o, &lem_, nullptr));
    }
    ~lem_engine() { lsdtt_gpu_lem_destroy(lem_); }
    lem_engine(const lem_engine&) = delete;
    lem_engine& operator=(const lem_engine&) = delete;

    // One timestep of z (host, updated in place); returns the step's
    // statistics (lsdtt_lem_step_stats).
    lsdtt_gpu_lem_stats step(std::vector<float>& z)
    {
        if (z.size() != grid_.cells()) throw std::invalid_argument("run_lem_step: dem size does not match the grid");
        zd_.from_host(z.data());
        lsdtt_gpu_lem_stats st{};
        check(lsdtt_gpu_lem_step(lem_, zd_.get(), &st, nullptr));
        z = zd_.to_host();
        return st;
    }

private:
    grid grid_;
    lsdtt_gpu_lem* lem_ = nullptr;
    device_buffer<float> zd_;
};

}  // namespace lsdtt_gb300_host
