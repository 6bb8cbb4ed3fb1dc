// lsdtt_flowinfo_gpu.hpp -- the GB300 D8 engine behind lsdtt3's abstract
// flow seam.
//
// Drop-in for src/cpu/lsdtt_flowinfo_cpu.hpp behind
//   class lsdtt_flow_base            (src/core/lsdtt_flow_base.hpp:126-491)
//   std::unique_ptr<lsdtt_flow_base>
//   make_flow_base(dem, mask, meta, options)   (:504-509, src/cpu/lsdtt_flow_base.cpp:170-183)
// Build it into lsdtt3 with the lsdtt3 include paths (src/core, src/utils,
// src/cpu), this repository's include/ and the CUDA runtime, and link
// liblsdtt_gb300.so. Construction uploads the DEM, builds every component on
// the GPU (lsdtt_gpu_flow_build) and mirrors the arrays to host memory once,
// so every const query is a plain host read: safe to call concurrently after
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
#include "lsdtt_gb300.h"        // this repository: include/

namespace lsdtt
{

class lsdtt_flowinfo_gpu final : public lsdtt_flow_base
{
public:
    lsdtt_flowinfo_gpu(const lsdtt_array2d_f& dem, const lsdtt_array2d_u8& mask, const lsdtt_raster_meta& meta,
                       const lsdtt_flowinfo_options& options = lsdtt_flowinfo_options{})
        : meta_(meta)
    {
        if (options.boundary_conditions.size() != 4)
            throw std::runtime_error(
                "lsdtt_flowinfo: boundary_conditions must have length 4 (north, east, south, west)");
        lsdtt_gpu_grid g{};
        g.n_rows = meta.n_rows;
        g.n_cols = meta.n_cols;
        g.cell_size = meta.cell_size;
        g.no_data_value = meta.no_data_value;
        std::memcpy(g.boundary_conditions, options.boundary_conditions.data(), 4);
        check(lsdtt_gpu_flow_create(&g, &flow_));
        const std::size_t n = static_cast<std::size_t>(meta.n_rows) * meta.n_cols;
        float* zd = nullptr;
        std::uint8_t* md = nullptr;
        std::int64_t* fd = nullptr;
        cuda(cudaMalloc(&zd, sizeof(float) * n));
        cuda(cudaMalloc(&md, n));
        cuda(cudaMemcpy(zd, dem.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
        cuda(cudaMemcpy(md, mask.data(), n, cudaMemcpyHostToDevice));
        if (!options.forced_outlet_flats.empty())
        {
            cuda(cudaMalloc(&fd, sizeof(std::int64_t) * options.forced_outlet_flats.size()));
            cuda(cudaMemcpy(fd, options.forced_outlet_flats.data(),
                            sizeof(std::int64_t) * options.forced_outlet_flats.size(), cudaMemcpyHostToDevice));
        }
        lsdtt_gpu_flow_options o{options.interior_nodata_is_outlet ? 1 : 0, options.require_acyclic_graph ? 1 : 0,
                                 options.build_topological_order ? 1 : 0, options.build_s_vector ? 1 : 0,
                                 options.allow_pits_as_outlets ? 1 : 0};
        const int st = lsdtt_gpu_flow_build(flow_, zd, md, &o, fd,
                                            static_cast<std::int64_t>(options.forced_outlet_flats.size()), nullptr);
        cudaFree(zd);
        cudaFree(md);
        cudaFree(fd);
        check(st);
        lsdtt_gpu_flow_view v{};
        check(lsdtt_gpu_flow_get_view(flow_, &v));
        mask_.assign(mask.data(), mask.data() + n);
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

    ~lsdtt_flowinfo_gpu() override { lsdtt_gpu_flow_destroy(flow_); }
    lsdtt_flowinfo_gpu(const lsdtt_flowinfo_gpu&) = delete;
    lsdtt_flowinfo_gpu& operator=(const lsdtt_flowinfo_gpu&) = delete;

    // ---- state ---------------------------------------------------------
    bool empty() const noexcept override { return n_valid_ == 0; }
    bool is_acyclic() const noexcept override { return acyclic_; }
    bool has_s_vector() const noexcept override { return has_sv_; }
    bool has_topological_order() const noexcept override { return has_topo_; }
    std::int64_t n_valid_cells() const noexcept override { return n_valid_; }
    std::size_t n_outlets() const noexcept override { return outlets_.size(); }
    std::size_t full_grid_size() const noexcept override { return mask_.size(); }
    const lsdtt_raster_meta& meta() const noexcept override { return meta_; }
    int n_rows() const noexcept override { return meta_.n_rows; }
    int n_cols() const noexcept override { return meta_.n_cols; }
    double cell_size() const noexcept override { return meta_.cell_size; }

    // ---- indexing ------------------------------------------------------
    bool in_bounds(int r, int c) const noexcept override
    {
        return r >= 0 && r < meta_.n_rows && c >= 0 && c < meta_.n_cols;
    }
    bool is_flat_in_range(std::int64_t f) const noexcept override
    {
        return f >= 0 && f < static_cast<std::int64_t>(mask_.size());
    }
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
    int row_from_flat(std::int64_t f) const override { require_range(f); return row_from_flat_unchecked(f); }
    int col_from_flat(std::int64_t f) const override { require_range(f); return col_from_flat_unchecked(f); }
    bool is_valid_cell(std::int64_t f) const noexcept override { return is_flat_in_range(f) && mask_[f] != 0; }
    bool is_valid_cell(int r, int c) const noexcept override { return in_bounds(r, c) && mask_[flat_index_unchecked(r, c)]; }

    // ---- receivers -------------------------------------------------------
    bool is_outlet_unchecked(std::int64_t f) const noexcept override { return receiver_[f] == k_outlet_receiver; }
    std::int64_t receiver_of_unchecked(std::int64_t f) const noexcept override { return receiver_[f]; }
    std::uint8_t receiver_dir_of_unchecked(std::int64_t f) const noexcept override { return dir_[f]; }
    std::uint8_t donor_count_of_unchecked(std::int64_t f) const noexcept override { return donors_[f]; }
    bool is_influenced_by_invalid(std::int64_t f) const override
    {
        require_valid(f);
        const int r = row_from_flat_unchecked(f), c = col_from_flat_unchecked(f);
        for (int dr = -1; dr <= 1; ++dr)
            for (int dc = -1; dc <= 1; ++dc)
                if ((dr || dc) && (!in_bounds(r + dr, c + dc) || !mask_[flat_index_unchecked(r + dr, c + dc)]))
                    return true;
        return false;
    }
    bool is_outlet(std::int64_t f) const override { require_valid(f); return is_outlet_unchecked(f); }
    std::int64_t receiver_of(std::int64_t f) const override { require_valid(f); return receiver_[f]; }
    std::uint8_t receiver_dir_of(std::int64_t f) const override { require_valid(f); return dir_[f]; }
    std::uint8_t donor_count_of(std::int64_t f) const override { require_valid(f); return donors_[f]; }

    // ---- s-vector --------------------------------------------------------
    std::int64_t s_vector_start_unchecked(std::int64_t f) const noexcept override { return start_[f]; }
    std::uint64_t s_vector_size_unchecked(std::int64_t f) const noexcept override { return size_[f]; }
    std::int64_t s_vector_start(std::int64_t f) const override { require_sv(f); return start_[f]; }
    std::uint64_t s_vector_size(std::int64_t f) const override { require_sv(f); return size_[f]; }
    lsdtt_flat_index_slice upslope_nodes(std::int64_t f) const override { require_sv(f); return upslope_nodes_unchecked(f); }
    lsdtt_flat_index_slice upslope_nodes(int r, int c) const override { return upslope_nodes(flat_index(r, c)); }
    lsdtt_flat_index_slice upslope_nodes_unchecked(std::int64_t f) const noexcept override
    {
        return lsdtt_flat_index_slice(svec_.data() + start_[f], static_cast<std::size_t>(size_[f]));
    }
    bool is_upslope_of(std::int64_t cand, std::int64_t target) const override
    {
        require_sv(cand);
        require_sv(target);
        return is_upslope_of_unchecked(cand, target);
    }
    bool is_upslope_of_unchecked(std::int64_t cand, std::int64_t target) const noexcept override
    {
        const std::int64_t a = start_[target], s = start_[cand];
        return s >= a && s < a + static_cast<std::int64_t>(size_[target]);
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
        if (!has_sv_ || !has_topo_)
            throw std::logic_error("get_sources_index_threshold: s_vector and topological_order must be built");
        std::vector<std::int64_t> out;
        for (const std::int64_t f : topo_)
        {
            if (static_cast<int>(size_[f]) < threshold) continue;
            bool above = false;
            for (const std::int64_t x : upslope_nodes_unchecked(f))
                if (x != f && receiver_[x] == f && static_cast<int>(size_[x]) >= threshold) { above = true; break; }
            if (!above) out.push_back(f);
        }
        return out;
    }

    // ---- rasters -----------------------------------------------------------
    lsdtt_raster_result get_d8_flow_direction_raster() const override
    {
        return raster([&](std::size_t i) { return static_cast<float>(dir_[i]); });
    }
    lsdtt_raster_result get_n_contributing_pixels_raster() const override
    {
        need_sv_raster();
        return raster([&](std::size_t i) { return static_cast<float>(size_[i]); });
    }
    lsdtt_raster_result get_n_contributing_pixels_exclude_outlet_raster() const override
    {
        need_sv_raster();
        return raster([&](std::size_t i) { return static_cast<float>(size_[i] > 0 ? size_[i] - 1 : 0); });
    }
    lsdtt_raster_result get_drainage_area_raster() const override
    {
        const double a = meta_.cell_size * meta_.cell_size;
        if (has_sv_) return raster([&](std::size_t i) { return static_cast<float>(static_cast<double>(size_[i]) * a); });
        const std::vector<double> acc = accumulate({});
        return raster([&](std::size_t i) { return static_cast<float>(acc[i]); });
    }
    lsdtt_raster_result get_drainage_area_exclude_outlet_raster() const override
    {
        need_sv_raster();
        const double a = meta_.cell_size * meta_.cell_size;
        return raster([&](std::size_t i) {
            return static_cast<float>(static_cast<double>(size_[i] > 0 ? size_[i] - 1 : 0) * a);
        });
    }

    // lsdtt_flowinfo::accumulate (not on the abstract seam): computed on the GPU.
    std::vector<double> accumulate(const std::vector<double>& weights) const
    {
        const std::size_t n = mask_.size();
        if (!weights.empty() && weights.size() != n)
            throw std::invalid_argument(
                "lsdtt_flowinfo::accumulate: cell_weights size must equal n_rows * n_cols");
        double* wd = nullptr;
        double* od = nullptr;
        cuda(cudaMalloc(&od, sizeof(double) * n));
        if (!weights.empty())
        {
            cuda(cudaMalloc(&wd, sizeof(double) * n));
            cuda(cudaMemcpy(wd, weights.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
        }
        const int st = lsdtt_gpu_flow_accumulate(flow_, wd, od, nullptr);
        std::vector<double> out(n);
        if (st == LSDTT_GPU_OK) cudaMemcpy(out.data(), od, sizeof(double) * n, cudaMemcpyDeviceToHost);
        cudaFree(wd);
        cudaFree(od);
        check(st);
        return out;
    }

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

    // Analysis rasters built on the stack: next on the GB300 engine.
    lsdtt_raster_result get_distance_from_outlet_raster() const override { not_yet("get_distance_from_outlet_raster"); }
    lsdtt_raster_result get_height_above_channel_raster(const std::vector<float>&, const std::vector<uint8_t>&,
                                                        int) const override
    {
        not_yet("get_height_above_channel_raster");
    }
    lsdtt_raster_result get_height_above_channel_mask_raster(const std::vector<float>&, const std::vector<uint8_t>&,
                                                             const std::vector<uint8_t>&) const override
    {
        not_yet("get_height_above_channel_mask_raster");
    }
    height_above_channel_donor_result get_height_above_channel_mask_donor_raster(
        const std::vector<float>&, const std::vector<uint8_t>&, const std::vector<uint8_t>&) const override
    {
        not_yet("get_height_above_channel_mask_donor_raster");
    }
    lsdtt_raster_result get_distance_to_channel_raster(int) const override { not_yet("get_distance_to_channel_raster"); }
    lsdtt_raster_result get_height_to_farthest_ridge_raster(const std::vector<float>&,
                                                            const std::vector<uint8_t>&) const override
    {
        not_yet("get_height_to_farthest_ridge_raster");
    }
    lsdtt_raster_result get_distance_to_farthest_ridge_raster() const override
    {
        not_yet("get_distance_to_farthest_ridge_raster");
    }
    lsdtt_raster_result get_downstream_path_sum_raster(const std::vector<float>&, const std::vector<uint8_t>&,
                                                       const std::vector<uint8_t>&) const override
    {
        not_yet("get_downstream_path_sum_raster");
    }
    lsdtt_raster_result get_upslope_sum_raster(const std::vector<float>&, const std::vector<uint8_t>&,
                                               bool) const override
    {
        not_yet("get_upslope_sum_raster");
    }
    lsdtt_raster_result get_upslope_mean_raster(const std::vector<float>&, const std::vector<uint8_t>&,
                                                bool) const override
    {
        not_yet("get_upslope_mean_raster");
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
    static void check(int st)
    {
        if (st == LSDTT_GPU_OK) return;
        const std::string msg = lsdtt_gpu_last_error();
        if (st == LSDTT_GPU_EINVAL && msg.find("forced outlet") != std::string::npos) throw std::invalid_argument(msg);
        throw std::runtime_error(msg);
    }
    static void cuda(cudaError_t e)
    {
        if (e != cudaSuccess) throw std::runtime_error(std::string("lsdtt_flowinfo_gpu: ") + cudaGetErrorString(e));
    }
    template <class T>
    static void pull(std::vector<T>& dst, const T* src, std::size_t n)
    {
        dst.resize(n);
        if (n) cuda(cudaMemcpy(dst.data(), src, sizeof(T) * n, cudaMemcpyDeviceToHost));
    }
    [[noreturn]] static void not_yet(const char* what)
    {
        throw std::logic_error(std::string("lsdtt_flowinfo_gpu::") + what + " is not available on the GB300 engine yet");
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
    void require_sv(std::int64_t f) const
    {
        require_valid(f);
        if (!has_sv_) throw std::runtime_error("lsdtt_flowinfo: s_vector was not built for this object");
    }
    void need_sv_raster() const
    {
        if (!has_sv_)
            throw std::runtime_error(
                "lsdtt_flowinfo: s_vector not built - set build_s_vector = true in lsdtt_flowinfo_options");
    }
    template <class F>
    lsdtt_raster_result raster(F value) const
    {
        lsdtt_raster_result r;
        r.meta = meta_;
        const std::size_t n = mask_.size();
        r.data.assign(n, static_cast<float>(meta_.no_data_value));
        r.mask.assign(n, 0u);
        for (std::size_t i = 0; i < n; ++i)
            if (mask_[i]) { r.data[i] = value(i); r.mask[i] = 1u; }
        return r;
    }
    static void write(const lsdtt_raster_result& r, const std::string& p, raster_output_format f)
    {
        lsdtt_data_loader loader;
        loader.write_full(r, p, f);
    }

    lsdtt_raster_meta meta_;
    lsdtt_gpu_flow* flow_ = nullptr;
    std::vector<std::uint8_t> mask_;
    std::vector<std::int64_t> receiver_, outlets_, topo_, svec_, start_;
    std::vector<std::uint8_t> dir_, donors_;
    std::vector<std::uint64_t> size_;
    std::int64_t n_valid_ = 0;
    bool acyclic_ = false, has_topo_ = false, has_sv_ = false;
};

}  // namespace lsdtt
