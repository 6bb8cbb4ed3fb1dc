// ref_shim.cpp -- test infrastructure only.
//
// A C-ABI wrapper around the reference lsdtt3 C++ implementation of the
// landscape-evolution hot path, compiled from the reference's own sources by
// oracle/Makefile (target `ref`) into oracle/_ref/liblsdtt_ref.so. It is the
// ground truth that the CPU restatement in oracle/lsdtt_oracle.cpp is checked
// against. Nothing in the product links or loads it.
//
// Every function returns 0 on success and 1 when the reference threw; the
// exception text is copied into `err` (NUL-terminated, truncated to errlen).

#include "lsdtt_flowgraph_cpu.hpp"
#include "lsdtt_flowinfo_cpu.hpp"
#include "lsdtt_raster_flow_preprocessing_cpu.hpp"
#include "lsdtt_stream_power_cpu.hpp"
#include "lsdtt_lem_cpu.hpp"
#include "lsdtt_raster_synthetic_surfaces_cpu.hpp"

#include <cstdint>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

using namespace lsdtt;

namespace
{

void put_err(char* err, int errlen, const char* what)
{
    if (!err || errlen <= 0) return;
    std::strncpy(err, what, static_cast<std::size_t>(errlen - 1));
    err[errlen - 1] = '\0';
}

lsdtt_raster_meta make_meta(int nr, int nc, double cell, double nodata)
{
    lsdtt_raster_meta m;
    m.n_rows = nr;
    m.n_cols = nc;
    m.cell_size = cell;
    m.no_data_value = nodata;
    return m;
}

lsdtt_raster_cpu make_raster(const float* z, const std::uint8_t* mask,
                             int nr, int nc, double cell, double nodata)
{
    const std::size_t n = static_cast<std::size_t>(nr) * nc;
    std::vector<float> d(z, z + n);
    std::vector<std::uint8_t> m(mask, mask + n);
    return lsdtt_raster_cpu(std::move(d), std::move(m), make_meta(nr, nc, cell, nodata));
}

lsdtt_array2d_f make_a2f(const float* z, int nr, int nc)
{
    lsdtt_array2d_f a(nr, nc, 0.0f);
    std::memcpy(a.data(), z, sizeof(float) * static_cast<std::size_t>(nr) * nc);
    return a;
}

lsdtt_array2d_u8 make_a2u8(const std::uint8_t* m, int nr, int nc)
{
    lsdtt_array2d_u8 a(nr, nc, std::uint8_t{0});
    std::memcpy(a.data(), m, static_cast<std::size_t>(nr) * nc);
    return a;
}

} // namespace

extern "C" {

// fill_pits(raster, min_slope, bc, n_threads, binary_heap)
// (src/cpu/lsdtt_raster_flow_preprocessing_cpu.hpp:191-199)
int ref_fill_pits(const float* z, const std::uint8_t* mask, int nr, int nc,
                  double cell, double nodata, const char* bc, float min_slope,
                  int radix_queue, float* out, char* err, int errlen)
{
    try
    {
        const lsdtt_raster_cpu r = make_raster(z, mask, nr, nc, cell, nodata);
        const lsdtt_raster_cpu f = fill_pits(
            r, min_slope, std::string(bc), 1,
            radix_queue ? priority_flood_queue_backend::radix_hybrid
                        : priority_flood_queue_backend::binary_heap);
        std::memcpy(out, f.get_data().data(), sizeof(float) * f.get_data().size());
        return 0;
    }
    catch (const std::exception& e) { put_err(err, errlen, e.what()); return 1; }
}

// lsdtt_flowinfo construction plus every component the byte-identity test
// pins (tests/cpp/test_flow_d8_identity.cpp:343-420). Output arrays are sized
// n = nr*nc by the caller (outlets/topo/s_vector: n entries of room).
// `weights` may be null (default dx^2 weights) and `accum` may be null.
int ref_flowinfo(const float* z, const std::uint8_t* mask, int nr, int nc,
                 double cell, double nodata, const char* bc,
                 int interior_nodata_is_outlet, int allow_pits_as_outlets,
                 int build_topo, int build_sv, int require_acyclic,
                 const std::int64_t* forced, std::int64_t n_forced, int n_threads,
                 std::int64_t* receiver, std::uint8_t* dir, std::uint8_t* donors,
                 std::int64_t* outlets, std::int64_t* n_outlets,
                 std::int64_t* topo, std::int64_t* n_topo,
                 std::int64_t* svec, std::int64_t* sv_start, std::uint64_t* sv_size,
                 std::int32_t* flags, const double* weights, double* accum,
                 char* err, int errlen)
{
    try
    {
        const std::int64_t n = static_cast<std::int64_t>(nr) * nc;
        lsdtt_flowinfo_options o;
        o.boundary_conditions = bc;
        o.interior_nodata_is_outlet = interior_nodata_is_outlet != 0;
        o.allow_pits_as_outlets = allow_pits_as_outlets != 0;
        o.build_topological_order = build_topo != 0;
        o.build_s_vector = build_sv != 0;
        o.require_acyclic_graph = require_acyclic != 0;
        o.n_threads = n_threads;
        if (forced && n_forced > 0) o.forced_outlet_flats.assign(forced, forced + n_forced);

        const lsdtt_flowinfo fi(make_a2f(z, nr, nc), make_a2u8(mask, nr, nc),
                                make_meta(nr, nc, cell, nodata), o);
        for (std::int64_t f = 0; f < n; ++f)
        {
            receiver[f] = fi.receiver_of_unchecked(f);
            dir[f] = fi.receiver_dir_of_unchecked(f);
            donors[f] = fi.donor_count_of_unchecked(f);
        }
        const auto& outs = fi.outlets();
        *n_outlets = static_cast<std::int64_t>(outs.size());
        std::memcpy(outlets, outs.data(), sizeof(std::int64_t) * outs.size());
        flags[0] = fi.has_topological_order() ? 1 : 0;
        flags[1] = fi.has_s_vector() ? 1 : 0;
        *n_topo = 0;
        if (fi.has_topological_order())
        {
            const auto& t = fi.topological_order();
            *n_topo = static_cast<std::int64_t>(t.size());
            std::memcpy(topo, t.data(), sizeof(std::int64_t) * t.size());
        }
        if (fi.has_s_vector())
        {
            std::int64_t pos = 0;
            for (const std::int64_t out : outs)
            {
                const auto slice = fi.upslope_nodes(out);
                std::memcpy(svec + pos, slice.data(), sizeof(std::int64_t) * slice.size());
                pos += static_cast<std::int64_t>(slice.size());
            }
            for (std::int64_t f = 0; f < n; ++f)
            {
                sv_start[f] = fi.s_vector_start_unchecked(f);
                sv_size[f] = fi.s_vector_size_unchecked(f);
            }
        }
        if (accum && fi.has_topological_order())
        {
            std::vector<double> w;
            if (weights) w.assign(weights, weights + n);
            const std::vector<double> a = fi.accumulate(w);
            std::memcpy(accum, a.data(), sizeof(double) * a.size());
        }
        return 0;
    }
    catch (const std::exception& e) { put_err(err, errlen, e.what()); return 1; }
}

// compute_d8_stream_power_incision on a flow object built the way run_lem_step
// builds it (src/cpu/lsdtt_lem_cpu.cpp:329-339).
int ref_stream_power(const float* z, const std::uint8_t* mask, int nr, int nc,
                     double cell, double nodata, const char* bc,
                     float K, float m, float n_exp, float dt,
                     float threshold_area, int divide_area_by_dx, float slope_clamp,
                     const float* k_field, float* out, char* err, int errlen)
{
    try
    {
        const lsdtt_raster_cpu dem = make_raster(z, mask, nr, nc, cell, nodata);
        lsdtt_flowinfo_options o;
        o.boundary_conditions = bc;
        o.interior_nodata_is_outlet = true;
        o.allow_pits_as_outlets = true;
        const lsdtt_flowinfo fi(dem.get_data_array(), dem.get_mask_array(), dem.get_meta(), o);
        std::vector<float> kf;
        if (k_field) kf.assign(k_field, k_field + static_cast<std::size_t>(nr) * nc);
        const lsdtt_raster_cpu r = compute_d8_stream_power_incision(
            dem, fi, K, m, n_exp, dt, threshold_area, divide_area_by_dx != 0,
            slope_clamp, 1, std::string(bc), kf, false, 1.0f);
        std::memcpy(out, r.get_data().data(), sizeof(float) * r.get_data().size());
        return 0;
    }
    catch (const std::exception& e) { put_err(err, errlen, e.what()); return 1; }
}

// run_lem_step with the hillslope stage switched off: D8 flow, stream power,
// uplift, boundary restore and statistics (src/cpu/lsdtt_lem_cpu.cpp:285-732).
// stats (6 floats): delta_max, delta_mean, max_local, p999_local,
// mean_erosion_rate, max_erosion_rate.
int ref_lem_step_fluvial(const float* z, const std::uint8_t* mask, int nr, int nc,
                         double cell, double nodata, const char* bc,
                         float dt, float K, float m, float n_exp, float U,
                         const std::int64_t* boundary_flats, std::int64_t n_bf,
                         float* out, float* stats, char* err, int errlen)
{
    try
    {
        const lsdtt_raster_cpu dem = make_raster(z, mask, nr, nc, cell, nodata);
        lsdtt_lem_options o;
        o.timestep = dt;
        o.erodibility = K;
        o.m_exponent = m;
        o.n_exponent = n_exp;
        o.uplift_rate = U;
        o.enable_hillslope_transport = false;
        o.boundary_conditions = bc;
        std::vector<std::int64_t> bf(boundary_flats, boundary_flats + n_bf);
        const auto res = run_lem_step(dem, o, bf, nullptr, nullptr, nullptr);
        std::memcpy(out, res.first.get_data().data(),
                    sizeof(float) * res.first.get_data().size());
        stats[0] = res.second.delta_max_elevation;
        stats[1] = res.second.delta_mean_elevation;
        stats[2] = res.second.max_local_elevation_change;
        stats[3] = res.second.p999_local_elevation_change;
        stats[4] = res.second.mean_erosion_rate;
        stats[5] = res.second.max_erosion_rate;
        return 0;
    }
    catch (const std::exception& e) { put_err(err, errlen, e.what()); return 1; }
}

// The lsdtt_flow_base query rasters of the reference's own lsdtt_flowinfo
// (src/cpu/lsdtt_flowinfo_cpu.cpp:2255-2965), with the same `kind` codes as
// oracle_flow_query.
int ref_flow_query(const float* z, const std::uint8_t* mask, int nr, int nc, double cell, double nodata,
                   const char* bc, int kind, const float* values, const std::uint8_t* vmask,
                   const std::uint8_t* cmask, int threshold, int include_self, float* out,
                   std::uint8_t* out_mask, std::int64_t* donor_out, char* err, int errlen)
{
    try
    {
        const std::size_t n = static_cast<std::size_t>(nr) * nc;
        lsdtt_flowinfo_options o;
        o.boundary_conditions = bc;
        o.allow_pits_as_outlets = true;
        const lsdtt_flowinfo fi(make_a2f(z, nr, nc), make_a2u8(mask, nr, nc), make_meta(nr, nc, cell, nodata), o);
        const std::vector<float> v(values ? values : z, (values ? values : z) + n);
        const std::vector<std::uint8_t> vm(vmask ? vmask : mask, (vmask ? vmask : mask) + n);
        const std::vector<std::uint8_t> cm(cmask ? cmask : mask, (cmask ? cmask : mask) + n);
        lsdtt_raster_result r;
        switch (kind)
        {
        case 0: r = fi.get_distance_from_outlet_raster(); break;
        case 1: r = fi.get_height_above_channel_raster(v, vm, threshold); break;
        case 2:
        {
            auto d = fi.get_height_above_channel_mask_donor_raster(v, vm, cm);
            r = std::move(d.height);
            if (donor_out) std::memcpy(donor_out, d.donor_flat.data(), sizeof(std::int64_t) * n);
            break;
        }
        case 3: r = fi.get_distance_to_channel_raster(threshold); break;
        case 4: r = fi.get_height_to_farthest_ridge_raster(v, vm); break;
        case 5: r = fi.get_distance_to_farthest_ridge_raster(); break;
        case 6: r = fi.get_downstream_path_sum_raster(v, vm, cm); break;
        case 7: r = fi.get_upslope_sum_raster(v, vm, include_self != 0); break;
        case 8: r = fi.get_upslope_mean_raster(v, vm, include_self != 0); break;
        default: put_err(err, errlen, "ref_flow_query: unknown kind"); return 1;
        }
        std::memcpy(out, r.data.data(), sizeof(float) * n);
        std::memcpy(out_mask, r.mask.data(), n);
        return 0;
    }
    catch (const std::exception& e) { put_err(err, errlen, e.what()); return 1; }
}

// The reference's own D-infinity lsdtt_flowgraph_cpu (flowgraph_cpu.cpp:
// 87-178, 423-662, 874-985, 988-1039) and compute_dinf_stream_power_incision
// (stream_power_cpu.cpp:329-602), with the outputs of oracle_dinf_*.
static lsdtt_flowgraph_cpu make_dinf(const float* z, const std::uint8_t* mask, int nr, int nc, double cell,
                                     double nodata, const char* bc, int interior_nodata_is_outlet)
{
    lsdtt_flowgraph_options o;
    o.boundary_conditions = bc;
    o.interior_nodata_is_outlet = interior_nodata_is_outlet != 0;
    o.method = lsdtt_flowgraph_method::d_infinity;
    return lsdtt_flowgraph_cpu(make_a2f(z, nr, nc), make_a2u8(mask, nr, nc), make_meta(nr, nc, cell, nodata), o);
}

int ref_dinf_graph(const float* z, const std::uint8_t* mask, int nr, int nc, double cell, double nodata,
                   const char* bc, int interior_nodata_is_outlet, std::int64_t* rec, float* w, std::uint8_t* nrec,
                   float* slope, float* bearing, std::uint8_t* donors, std::int64_t* topo, std::int64_t* n_topo,
                   char* err, int errlen)
{
    try
    {
        const lsdtt_flowgraph_cpu g = make_dinf(z, mask, nr, nc, cell, nodata, bc, interior_nodata_is_outlet);
        const std::int64_t n = static_cast<std::int64_t>(nr) * nc;
        for (std::int64_t f = 0; f < n; ++f)
        {
            const std::int64_t k = g.n_receivers(f);
            nrec[f] = static_cast<std::uint8_t>(k);
            for (int j = 0; j < 2; ++j)
            {
                rec[2 * f + j] = j < k ? g.receiver_index_at(f, j) : -1;
                w[2 * f + j] = j < k ? g.receiver_weight_at(f, j) : 0.0f;
            }
            donors[f] = g.donor_count()[static_cast<std::size_t>(f)];
        }
        const lsdtt_raster_result s = g.dinf_slopes();
        const lsdtt_raster_result d = g.dinf_flow_direction();
        std::memcpy(slope, s.data.data(), sizeof(float) * static_cast<std::size_t>(n));
        std::memcpy(bearing, d.data.data(), sizeof(float) * static_cast<std::size_t>(n));
        const auto& t = g.topological_order();
        *n_topo = static_cast<std::int64_t>(t.size());
        std::memcpy(topo, t.data(), sizeof(std::int64_t) * t.size());
        return 0;
    }
    catch (const std::exception& e) { put_err(err, errlen, e.what()); return 1; }
}

int ref_dinf_accumulate(const float* z, const std::uint8_t* mask, int nr, int nc, double cell, double nodata,
                        const char* bc, const double* weights, double* out, char* err, int errlen)
{
    try
    {
        const lsdtt_flowgraph_cpu g = make_dinf(z, mask, nr, nc, cell, nodata, bc, 1);
        const std::size_t n = static_cast<std::size_t>(nr) * nc;
        const std::vector<double> w = weights ? std::vector<double>(weights, weights + n) : std::vector<double>{};
        const std::vector<double> a = g.accumulate(w);
        std::memcpy(out, a.data(), sizeof(double) * n);
        return 0;
    }
    catch (const std::exception& e) { put_err(err, errlen, e.what()); return 1; }
}

int ref_dinf_stream_power(const float* z, const std::uint8_t* mask, int nr, int nc, double cell, double nodata,
                          const char* bc, float K, float m, float n, float dt, float threshold_area,
                          int divide_area_by_dx, float slope_clamp, float* out, char* err, int errlen)
{
    try
    {
        const lsdtt_flowgraph_cpu g = make_dinf(z, mask, nr, nc, cell, nodata, bc, 1);
        const lsdtt_raster_cpu dem = make_raster(z, mask, nr, nc, cell, nodata);
        const lsdtt_raster_cpu r = compute_dinf_stream_power_incision(dem, g, K, m, n, dt, threshold_area,
                                                                      divide_area_by_dx != 0, slope_clamp, 1, 1, bc);
        std::memcpy(out, r.get_data().data(), sizeof(float) * static_cast<std::size_t>(nr) * nc);
        return 0;
    }
    catch (const std::exception& e) { put_err(err, errlen, e.what()); return 1; }
}

// build_boundary_flats (src/cpu/lsdtt_lem_cpu.cpp:735-808). Returns the count;
// `out` has room for nr*nc entries.
std::int64_t ref_boundary_flats(const std::uint8_t* mask, int nr, int nc, const char* bc,
                                std::int64_t* out)
{
    std::vector<float> d(static_cast<std::size_t>(nr) * nc, 0.0f);
    std::vector<std::uint8_t> mk(mask, mask + static_cast<std::size_t>(nr) * nc);
    const lsdtt_raster_cpu r(std::move(d), std::move(mk), make_meta(nr, nc, 1.0, -9999.0));
    const auto v = build_boundary_flats(r, std::string(bc));
    std::memcpy(out, v.data(), sizeof(std::int64_t) * v.size());
    return static_cast<std::int64_t>(v.size());
}

// generate_uniform_random_noise_surface(meta, seed, lo, hi) followed by
// superimpose_open_boundary_gradient(bc, slope)
// (src/cpu/lsdtt_raster_synthetic_surfaces_cpu.cpp:359-459).
int ref_noise_tilt_surface(int nr, int nc, double cell, int seed, double lo, double hi,
                           const char* bc, float slope, float* out, char* err, int errlen)
{
    try
    {
        const lsdtt_raster_meta meta = make_meta(nr, nc, cell, -9999.0);
        lsdtt_raster_cpu r = generate_uniform_random_noise_surface(meta, seed, lo, hi, 1);
        r = superimpose_open_boundary_gradient(r, std::string(bc), slope);
        std::memcpy(out, r.get_data().data(), sizeof(float) * r.get_data().size());
        return 0;
    }
    catch (const std::exception& e) { put_err(err, errlen, e.what()); return 1; }
}

} // extern "C"
