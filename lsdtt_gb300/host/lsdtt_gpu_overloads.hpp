// lsdtt_gpu_overloads.hpp -- the GB300 overloads at lsdtt3's fill,
// stream-power and LEM seams, in the reference's own types.
//
// The reference's LEM path bypasses the abstract flow seam: run_lem_step
// constructs the concrete lsdtt_flowinfo (src/cpu/lsdtt_lem_cpu.cpp:334-339)
// and compute_d8_stream_power_incision takes `const lsdtt_flowinfo&`
// (src/cpu/lsdtt_stream_power_cpu.hpp:74-89). These overloads give the same
// calls on the GB300 engine:
//
//   compute_d8_stream_power_incision(dem, const lsdtt_flowinfo_gpu&, ...)
//       same signature and defaults as stream_power_cpu.hpp:74-89;
//   fill_pits_gpu(raster, min_slope, bc)
//       fill_pits(raster, min_slope, bc, n_threads, backend),
//       raster_flow_preprocessing_cpu.hpp:191-199;
//   run_lem_step_gpu(dem, opts, boundary_flats)
//       run_lem_step (lem_cpu.hpp:223-232) for the configurations the GPU
//       step covers: D8 fluvial erosion (scalar K) in the coupled regime,
//       hillslopes off or "roering_implicit" (linear, or the Roering law with
//       enable_nonlinear_hillslopes), uplift, base-level fall.
//
// A caller switches on get_compute_backend() (backend_factory.hpp:115-116)
// at these three call sites. Options the GPU path does not implement throw
// std::invalid_argument naming the option, never a silent CPU run.
// Compile with the lsdtt3 include paths (src/core, src/utils, src/cpu), this
// repository's include/ and lsdtt_gb300/host/, and link liblsdtt_gb300.so.
#pragma once

#include <string>
#include <utility>
#include <vector>

#include "gb300_engine.hpp"
#include "lsdtt_flowinfo_gpu.hpp"
#include "lsdtt_lem_cpu.hpp"     // reference: src/cpu
#include "lsdtt_raster_cpu.hpp"  // reference: src/cpu

namespace lsdtt
{

namespace gb300_detail
{
inline lsdtt_gb300_host::grid geometry(const lsdtt_raster_meta& meta, const std::string& bc)
{
    lsdtt_gb300_host::grid g;
    g.n_rows = meta.n_rows;
    g.n_cols = meta.n_cols;
    g.cell_size = meta.cell_size;
    g.no_data_value = meta.no_data_value;
    g.boundary_conditions = bc;
    return g;
}

[[noreturn]] inline void unsupported(const std::string& where, const std::string& what)
{
    throw std::invalid_argument(where + ": " + what + " is not available on the GB300 path");
}
}  // namespace gb300_detail

inline lsdtt_raster_cpu compute_d8_stream_power_incision(
    const lsdtt_raster_cpu& dem, const lsdtt_flowinfo_gpu& flow, float K, float m, float n, float dt,
    float incision_threshold_area, bool divide_area_by_dx, float slope_clamp,
    int drainage_area_moving_average_kernel_size_pixels = 1, const std::string& boundary_conditions = "",
    const std::vector<float>& erodibility_field = {}, bool multiply_stream_power_term_by_w_over_dx = false,
    float channel_width_w = 1.0f)
{
    (void)boundary_conditions;  // only the area smoothing reads it, and it is the identity at kernel 1
    (void)channel_width_w;
    const char* who = "compute_d8_stream_power_incision";
    if (drainage_area_moving_average_kernel_size_pixels != 1)
        gb300_detail::unsupported(who, "drainage-area smoothing (kernel size != 1)");
    if (multiply_stream_power_term_by_w_over_dx) gb300_detail::unsupported(who, "the w/dx stream-power factor");
    const std::vector<float>& z = dem.get_data();
    if (z.size() != flow.full_grid_size())
        throw std::invalid_argument(std::string(who) + ": dem and flow grids differ in size");
    std::vector<float> out = lsdtt_gb300_host::stream_power_d8(flow.engine(), z.data(), K, m, n, dt,
                                                               incision_threshold_area, divide_area_by_dx,
                                                               slope_clamp, erodibility_field);
    std::vector<uint8_t> mask = dem.get_mask();
    return lsdtt_raster_cpu(std::move(out), std::move(mask), dem.get_meta());
}

inline lsdtt_raster_cpu fill_pits_gpu(const lsdtt_raster_cpu& raster, float min_slope,
                                      const std::string& boundary_conditions = "oooo")
{
    const lsdtt_raster_meta& meta = raster.get_meta();
    std::vector<float> out = lsdtt_gb300_host::fill_pits(gb300_detail::geometry(meta, boundary_conditions),
                                                         raster.get_data().data(), raster.get_mask().data(),
                                                         min_slope);
    std::vector<uint8_t> mask = raster.get_mask();
    return lsdtt_raster_cpu(std::move(out), std::move(mask), meta);
}

inline std::pair<lsdtt_raster_cpu, lsdtt_lem_step_stats> run_lem_step_gpu(
    const lsdtt_raster_cpu& dem, const lsdtt_lem_options& opts, const std::vector<std::int64_t>& boundary_flats)
{
    const char* who = "run_lem_step_gpu";
    if (!opts.enable_d8_fluvial_erosion) gb300_detail::unsupported(who, "a step without D8 fluvial erosion");
    if (opts.enable_dinf_fluvial_erosion) gb300_detail::unsupported(who, "D-infinity fluvial erosion");
    if (!opts.erodibility_field.empty()) gb300_detail::unsupported(who, "a per-pixel erodibility field");
    if (opts.drainage_area_moving_average_kernel_size_pixels != 1)
        gb300_detail::unsupported(who, "drainage-area smoothing (kernel size != 1)");
    if (opts.multiply_stream_power_term_by_w_over_dx) gb300_detail::unsupported(who, "the w/dx stream-power factor");
    if (!opts.explicit_channel_mask.empty() ||
        resolve_hillslope_coupling_regime(opts.coupling_regime, opts.incision_threshold_area, false) !=
            hillslope_coupling_regime::coupled)
        gb300_detail::unsupported(who, "the channels-as-boundaries regime");
    if (opts.enable_hillslope_transport && opts.hillslope_transport_model != "roering_implicit")
        gb300_detail::unsupported(who, "hillslope model '" + opts.hillslope_transport_model + "'");
    if (opts.compute_erosion_rate_field) gb300_detail::unsupported(who, "the per-pixel erosion-rate field");
    if (boundary_flats != build_boundary_flats(dem, opts.boundary_conditions))
        gb300_detail::unsupported(who, "a boundary_flats list other than build_boundary_flats(dem, bc)");

    lsdtt_gpu_lem_options o{};
    o.timestep = opts.timestep;
    o.erodibility = opts.erodibility;
    o.m_exponent = opts.m_exponent;
    o.n_exponent = opts.n_exponent;
    o.uplift_rate = opts.enable_uplift ? opts.uplift_rate : 0.0f;
    o.hillslope_diffusivity = opts.hillslope_diffusivity;
    o.slope_clamp = opts.slope_clamp;
    o.baselevel_fall_rate = opts.baselevel_fall_rate;
    o.fill_min_slope = 0.0f;  // run_lem_step does not fill
    o.enable_hillslope = opts.enable_hillslope_transport ? 1 : 0;
    o.divide_area_by_dx = opts.divide_area_by_dx ? 1 : 0;
    o.hillslope_rel_tol = 1e-8;
    o.hillslope_max_iter = 4000;
    o.hillslope_nonlinear = opts.enable_nonlinear_hillslopes ? 1 : 0;
    o.critical_slope = opts.critical_hillslope_slope;

    const lsdtt_raster_meta& meta = dem.get_meta();
    lsdtt_gb300_host::lem_engine lem(gb300_detail::geometry(meta, opts.boundary_conditions),
                                     dem.get_mask().data(), o);
    std::vector<float> z = dem.get_data();
    const lsdtt_gpu_lem_stats s = lem.step(z);
    lsdtt_lem_step_stats stats{};
    stats.delta_max_elevation = s.delta_max_elevation;
    stats.delta_mean_elevation = s.delta_mean_elevation;
    stats.max_local_elevation_change = s.max_local_elevation_change;
    stats.p999_local_elevation_change = s.p999_local_elevation_change;
    stats.mean_erosion_rate = s.mean_erosion_rate;
    stats.max_erosion_rate = s.max_erosion_rate;
    std::vector<uint8_t> mask = dem.get_mask();
    return {lsdtt_raster_cpu(std::move(z), std::move(mask), meta), stats};
}

}  // namespace lsdtt
