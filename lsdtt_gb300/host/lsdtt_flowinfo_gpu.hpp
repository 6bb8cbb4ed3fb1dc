// lsdtt_flowinfo_gpu.hpp -- the GB300 D8 engine behind lsdtt3's abstract
// flow seam.
//
// Drop-in for src/cpu/lsdtt_flowinfo_cpu.hpp behind
//   class lsdtt_flow_base            (src/core/lsdtt_flow_base.hpp:126-491)
//   std::unique_ptr<lsdtt_flow_base>
//   make_flow_base(dem, mask, meta, options)   (:504-509, src/cpu/lsdtt_flow_base.cpp:170-183)
// Build it into lsdtt3 with the lsdtt3 include paths (src/core, src/utils,
// src/cpu), this repository's include/ and lsdtt_gb300/host/, and the CUDA
// runtime, and link liblsdtt_gb300.so. It adapts the reference-free engine of
// gb300_engine.hpp (lsdtt_gb300_host::flow_engine) to the reference's types:
// construction uploads the DEM, builds every component on the GPU
// (lsdtt_gpu_flow_build) and mirrors the arrays to host memory once, so every
// const query is a plain host read: safe to call concurrently after
// construction, and upslope_nodes() slices stay valid for the engine's
// lifetime (flow_base.hpp:56-57, 198-204). Errors are thrown as the
// reference throws them (std::runtime_error / std::invalid_argument with the
// reference's messages). Analysis rasters that are not on the GPU yet throw
// std::logic_error.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "lsdtt_flow_base.hpp"  // reference: src/core
#include "gb300_engine.hpp"     // this repository: lsdtt_gb300/host/ (with include/)

namespace lsdtt
{

class lsdtt_flowinfo_gpu final : public lsdtt_flow_base
{
public:
    lsdtt_flowinfo_gpu(const lsdtt_array2d_f& dem, const lsdtt_array2d_u8& mask, const lsdtt_raster_meta& meta,
                       const lsdtt_flowinfo_options& options = lsdtt_flowinfo_options{})
        : meta_(meta), engine_(geometry(meta, options), dem.data(), mask.data(), engine_options(options))
    {
    }

    // The engine under the adapter (the stream-power and LEM overloads of
    // lsdtt_gpu_overloads.hpp run on it).
    const lsdtt_gb300_host::flow_engine& engine() const noexcept { return engine_; }

    ~lsdtt_flowinfo_gpu() override = default;
    lsdtt_flowinfo_gpu(const lsdtt_flowinfo_gpu&) = delete;
    lsdtt_flowinfo_gpu& operator=(const lsdtt_flowinfo_gpu&) = delete;

    // ---- state ---------------------------------------------------------
    bool empty() const noexcept override { return engine_.empty(); }
    bool is_acyclic() const noexcept override { return engine_.is_acyclic(); }
    bool has_s_vector() const noexcept override { return engine_.has_s_vector(); }
    bool has_topological_order() const noexcept override { return engine_.has_topological_order(); }
    std::int64_t n_valid_cells() const noexcept override { return engine_.n_valid_cells(); }
    std::size_t n_outlets() const noexcept override { return engine_.outlets().size(); }
    std::size_t full_grid_size() const noexcept override { return engine_.full_grid_size(); }
    const lsdtt_raster_meta& meta() const noexcept override { return meta_; }
    int n_rows() const noexcept override { return meta_.n_rows; }
    int n_cols() const noexcept override { return meta_.n_cols; }
    double cell_size() const noexcept override { return meta_.cell_size; }

    // ---- indexing ------------------------------------------------------
    bool in_bounds(int r, int c) const noexcept override
    {
        return r >= 0 && r < meta_.n_rows && c >= 0 && c < meta_.n_cols;
    }
    bool is_flat_in_range(std::int64_t f) const noexcept override { return engine_.is_flat_in_range(f); }
    std::int64_t flat_index_unchecked(int r, int c) const noexcept override
    {
        return static_cast<std::int64_t>(r) * meta_.n_cols + c;
    }
    int row_from_flat_unchecked(std::int64_t f) const noexcept override { return static_cast<int>(f / meta_.n_cols); }
    int col_from_flat_unchecked(std::int64_t f) const noexcept override { return static_cast<int>(f % meta_.n_cols); }
    std::int64_t flat_index(int r, int c) const override
    {
        if (!in_bounds(r, c)) throw std::out_of_range("lsdtt_flowinfo: row/col out of range");
        return flat_index_unchecked(r, c);
    }
    int row_from_flat(std::int64_t f) const override { return engine_.row_from_flat(f); }
    int col_from_flat(std::int64_t f) const override { return engine_.col_from_flat(f); }
    bool is_valid_cell(std::int64_t f) const noexcept override { return engine_.is_valid_cell(f); }
    bool is_valid_cell(int r, int c) const noexcept override
    {
        return in_bounds(r, c) && engine_.is_valid_cell(flat_index_unchecked(r, c));
    }

    // ---- receivers -------------------------------------------------------
    bool is_outlet_unchecked(std::int64_t f) const noexcept override
    {
        return engine_.receivers()[f] == k_outlet_receiver;
    }
    std::int64_t receiver_of_unchecked(std::int64_t f) const noexcept override { return engine_.receivers()[f]; }
    std::uint8_t receiver_dir_of_unchecked(std::int64_t f) const noexcept override { return engine_.directions()[f]; }
    std::uint8_t donor_count_of_unchecked(std::int64_t f) const noexcept override { return engine_.donor_counts()[f]; }
    bool is_influenced_by_invalid(std::int64_t f) const override
    {
        (void)engine_.receiver_of(f);  // the reference's range and validity checks
        const int r = row_from_flat_unchecked(f), c = col_from_flat_unchecked(f);
        for (int dr = -1; dr <= 1; ++dr)
            for (int dc = -1; dc <= 1; ++dc)
                if ((dr || dc) && (!in_bounds(r + dr, c + dc) || !engine_.is_valid_cell(flat_index_unchecked(r + dr, c + dc))))
                    return true;
        return false;
    }
    bool is_outlet(std::int64_t f) const override { return engine_.is_outlet(f); }
    std::int64_t receiver_of(std::int64_t f) const override { return engine_.receiver_of(f); }
    std::uint8_t receiver_dir_of(std::int64_t f) const override { return engine_.receiver_dir_of(f); }
    std::uint8_t donor_count_of(std::int64_t f) const override { return engine_.donor_count_of(f); }

    // ---- s-vector --------------------------------------------------------
    std::int64_t s_vector_start_unchecked(std::int64_t f) const noexcept override { return start()[f]; }
    std::uint64_t s_vector_size_unchecked(std::int64_t f) const noexcept override { return size()[f]; }
    std::int64_t s_vector_start(std::int64_t f) const override { return engine_.s_vector_start(f); }
    std::uint64_t s_vector_size(std::int64_t f) const override { return engine_.s_vector_size(f); }
    lsdtt_flat_index_slice upslope_nodes(std::int64_t f) const override
    {
        const auto s = engine_.upslope_nodes(f);
        return lsdtt_flat_index_slice(s.first, s.second);
    }
    lsdtt_flat_index_slice upslope_nodes(int r, int c) const override { return upslope_nodes(flat_index(r, c)); }
    lsdtt_flat_index_slice upslope_nodes_unchecked(std::int64_t f) const noexcept override
    {
        return lsdtt_flat_index_slice(svec().data() + start()[f], static_cast<std::size_t>(size()[f]));
    }
    bool is_upslope_of(std::int64_t cand, std::int64_t target) const override
    {
        return engine_.is_upslope_of(cand, target);
    }
    bool is_upslope_of_unchecked(std::int64_t cand, std::int64_t target) const noexcept override
    {
        const std::int64_t a = start()[target], s = start()[cand];
        return s >= a && s < a + static_cast<std::int64_t>(size()[target]);
    }
    void for_each_upslope_node(std::int64_t f, const std::function<void(std::int64_t)>& fn) const override
    {
        for (const std::int64_t x : upslope_nodes(f)) fn(x);
    }
    void for_each_upslope_node_unchecked(std::int64_t f, const std::function<void(std::int64_t)>& fn) const noexcept override
    {
        for (const std::int64_t x : upslope_nodes_unchecked(f)) fn(x);
    }
    std::vector<std::int64_t> get_sources_index_threshold(int threshold) const override
    {
        if (threshold <= 0) throw std::invalid_argument("get_sources_index_threshold: threshold must be positive");
        if (!engine_.has_s_vector() || !engine_.has_topological_order())
            throw std::logic_error("get_sources_index_threshold: s_vector and topological_order must be built");
        std::vector<std::int64_t> out;
        const auto& rec = engine_.receivers();
        for (const std::int64_t f : engine_.topological_order())
        {
            if (static_cast<int>(size()[f]) < threshold) continue;
            bool above = false;
            for (const std::int64_t x : upslope_nodes_unchecked(f))
                if (x != f && rec[x] == f && static_cast<int>(size()[x]) >= threshold) { above = true; break; }
            if (!above) out.push_back(f);
        }
        return out;
    }

    // ---- rasters -----------------------------------------------------------
    lsdtt_raster_result get_d8_flow_direction_raster() const override
    {
        return raster([&](std::size_t i) { return static_cast<float>(engine_.directions()[i]); });
    }
    lsdtt_raster_result get_n_contributing_pixels_raster() const override
    {
        need_sv_raster();
        return raster([&](std::size_t i) { return static_cast<float>(size()[i]); });
    }
    lsdtt_raster_result get_n_contributing_pixels_exclude_outlet_raster() const override
    {
        need_sv_raster();
        return raster([&](std::size_t i) { return static_cast<float>(size()[i] > 0 ? size()[i] - 1 : 0); });
    }
    lsdtt_raster_result get_drainage_area_raster() const override
    {
        const double a = meta_.cell_size * meta_.cell_size;
        if (engine_.has_s_vector())
            return raster([&](std::size_t i) { return static_cast<float>(static_cast<double>(size()[i]) * a); });
        const std::vector<double> acc = accumulate({});
        return raster([&](std::size_t i) { return static_cast<float>(acc[i]); });
    }
    lsdtt_raster_result get_drainage_area_exclude_outlet_raster() const override
    {
        need_sv_raster();
        const double a = meta_.cell_size * meta_.cell_size;
        return raster([&](std::size_t i) {
            return static_cast<float>(static_cast<double>(size()[i] > 0 ? size()[i] - 1 : 0) * a);
        });
    }

    // lsdtt_flowinfo::accumulate (not on the abstract seam): computed on the GPU.
    std::vector<double> accumulate(const std::vector<double>& weights) const { return engine_.accumulate(weights); }

    // Output writers go through the reference's own GDAL loader.
    void write_d8_flow_direction_raster(const std::string& p, raster_output_format f) const override
    {
        write(get_d8_flow_direction_raster(), p, f);
    }
    void write_n_contributing_pixels_raster(const std::string& p, raster_output_format f) const override
    {
        write(get_n_contributing_pixels_raster(), p, f);
    }
    void write_n_contributing_pixels_exclude_outlet_raster(const std::string& p, raster_output_format f) const override
    {
        write(get_n_contributing_pixels_exclude_outlet_raster(), p, f);
    }
    void write_drainage_area_raster(const std::string& p, raster_output_format f) const override
    {
        write(get_drainage_area_raster(), p, f);
    }
    void write_drainage_area_exclude_outlet_raster(const std::string& p, raster_output_format f) const override
    {
        write(get_drainage_area_exclude_outlet_raster(), p, f);
    }

    // Analysis rasters built on the stack (flowinfo_cpu.cpp:2255-2965), on the GPU.
    lsdtt_raster_result get_distance_from_outlet_raster() const override { return query(0); }
    lsdtt_raster_result get_height_above_channel_raster(const std::vector<float>& elev,
                                                        const std::vector<uint8_t>& elev_mask,
                                                        int threshold_contributing_pixels) const override
    {
        return query(1, elev, elev_mask, {}, threshold_contributing_pixels);
    }
    lsdtt_raster_result get_height_above_channel_mask_raster(const std::vector<float>& elev,
                                                             const std::vector<uint8_t>& elev_mask,
                                                             const std::vector<uint8_t>& channel_mask) const override
    {
        return query(2, elev, elev_mask, channel_mask);
    }
    height_above_channel_donor_result get_height_above_channel_mask_donor_raster(
        const std::vector<float>& elev, const std::vector<uint8_t>& elev_mask,
        const std::vector<uint8_t>& channel_mask) const override
    {
        auto r = engine_.query(2, elev, elev_mask, channel_mask);
        height_above_channel_donor_result out;
        out.height = as_raster(std::move(r));
        out.donor_flat = std::move(r.donor);
        return out;
    }
    lsdtt_raster_result get_distance_to_channel_raster(int threshold_contributing_pixels) const override
    {
        return query(3, {}, {}, {}, threshold_contributing_pixels);
    }
    lsdtt_raster_result get_height_to_farthest_ridge_raster(const std::vector<float>& elev,
                                                            const std::vector<uint8_t>& elev_mask) const override
    {
        return query(4, elev, elev_mask);
    }
    lsdtt_raster_result get_distance_to_farthest_ridge_raster() const override { return query(5); }
    lsdtt_raster_result get_downstream_path_sum_raster(const std::vector<float>& values,
                                                       const std::vector<uint8_t>& valid_mask,
                                                       const std::vector<uint8_t>& sink_mask) const override
    {
        return query(6, values, valid_mask, sink_mask);
    }
    lsdtt_raster_result get_upslope_sum_raster(const std::vector<float>& values, const std::vector<uint8_t>& valid_mask,
                                               bool include_self) const override
    {
        return query(7, values, valid_mask, {}, 1, include_self);
    }
    lsdtt_raster_result get_upslope_mean_raster(const std::vector<float>& values, const std::vector<uint8_t>& valid_mask,
                                                bool include_self) const override
    {
        return query(8, values, valid_mask, {}, 1, include_self);
    }
    void write_flow_lines(const std::string&, vector_output_format, const std::string&, bool) const override
    {
        not_yet("write_flow_lines");
    }
    void print_arcmap_d8_flowdirection(const std::string&, raster_output_format) const override
    {
        not_yet("print_arcmap_d8_flowdirection");
    }

private:
    static lsdtt_gb300_host::grid geometry(const lsdtt_raster_meta& meta, const lsdtt_flowinfo_options& o)
    {
        lsdtt_gb300_host::grid g;
        g.n_rows = meta.n_rows;
        g.n_cols = meta.n_cols;
        g.cell_size = meta.cell_size;
        g.no_data_value = meta.no_data_value;
        g.boundary_conditions = o.boundary_conditions;
        return g;
    }
    static lsdtt_gb300_host::flow_options engine_options(const lsdtt_flowinfo_options& o)
    {
        lsdtt_gb300_host::flow_options e;
        e.interior_nodata_is_outlet = o.interior_nodata_is_outlet;
        e.require_acyclic_graph = o.require_acyclic_graph;
        e.build_topological_order = o.build_topological_order;
        e.build_s_vector = o.build_s_vector;
        e.allow_pits_as_outlets = o.allow_pits_as_outlets;
        e.forced_outlet_flats = o.forced_outlet_flats;
        return e;
    }
    // Host mirrors without the per-call check (the unchecked queries).
    const std::vector<std::int64_t>& svec() const noexcept { return sv_or_empty(&lsdtt_gb300_host::flow_engine::s_vector); }
    const std::vector<std::int64_t>& start() const noexcept
    {
        return sv_or_empty(&lsdtt_gb300_host::flow_engine::s_vector_starts);
    }
    const std::vector<std::uint64_t>& size() const noexcept
    {
        static const std::vector<std::uint64_t> none;
        return engine_.has_s_vector() ? engine_.s_vector_sizes() : none;
    }
    const std::vector<std::int64_t>& sv_or_empty(
        const std::vector<std::int64_t>& (lsdtt_gb300_host::flow_engine::*get)() const) const noexcept
    {
        static const std::vector<std::int64_t> none;
        return engine_.has_s_vector() ? (engine_.*get)() : none;
    }
    lsdtt_raster_result as_raster(lsdtt_gb300_host::flow_engine::raster_out&& r) const
    {
        lsdtt_raster_result out;
        out.meta = meta_;
        out.data = std::move(r.data);
        out.mask = std::move(r.mask);
        return out;
    }
    lsdtt_raster_result query(int kind, const std::vector<float>& v = {}, const std::vector<uint8_t>& vm = {},
                              const std::vector<uint8_t>& cm = {}, int threshold = 1, bool include_self = true) const
    {
        return as_raster(engine_.query(kind, v, vm, cm, threshold, include_self));
    }
    [[noreturn]] static void not_yet(const char* what)
    {
        throw std::logic_error(std::string("lsdtt_flowinfo_gpu::") + what + " is not available on the GB300 engine yet");
    }
    void need_sv_raster() const
    {
        if (!engine_.has_s_vector())
            throw std::runtime_error(
                "lsdtt_flowinfo: s_vector not built - set build_s_vector = true in lsdtt_flowinfo_options");
    }
    template <class F>
    lsdtt_raster_result raster(F value) const
    {
        lsdtt_raster_result r;
        r.meta = meta_;
        const std::size_t n = engine_.full_grid_size();
        r.data.assign(n, static_cast<float>(meta_.no_data_value));
        r.mask.assign(n, 0u);
        for (std::size_t i = 0; i < n; ++i)
            if (engine_.is_valid_cell(static_cast<std::int64_t>(i))) { r.data[i] = value(i); r.mask[i] = 1u; }
        return r;
    }
    static void write(const lsdtt_raster_result& r, const std::string& p, raster_output_format f)
    {
        lsdtt_data_loader loader;
        loader.write_full(r, p, f);
    }

    lsdtt_raster_meta meta_;
    lsdtt_gb300_host::flow_engine engine_;
};

}  // namespace lsdtt
