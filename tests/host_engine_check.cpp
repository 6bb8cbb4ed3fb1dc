// Driver for tests/test_gpu_host_engine.py: runs the C++ host layer
// (lsdtt_gb300/host/gb300_engine.hpp) on one surface and writes every output
// as a raw little-endian file for the test to compare with the oracle.
//
//   host_engine_check <dir>
//
// <dir>/meta.txt: n_rows n_cols cell_size bc min_slope K m n dt U D
// <dir>/z.f32 (the surface to fill), <dir>/f.f32 (the surface to route: the
// oracle's fill of z), <dir>/mask.u8, <dir>/w.f64 (accumulation weights).
// Writes filled.f32, receiver.i64, direction.u8, donors.u8, outlets.i64,
// topo.i64, svec.i64, start.i64, size.u64, area.f64, weighted.f64, sp.f32,
// lem.f32, lem_stats.f32, upslope.i64 (for cells 0, 1, 2, ...: the slice
// length then its cells), q_dist.f32 / q_dist_mask.u8 (distance from the
// outlet), q_upsum.f32 (upslope sum of the weights as float) and
// errors.txt (one line per exception probe).
#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "gb300_engine.hpp"

namespace H = lsdtt_gb300_host;

template <class T>
static std::vector<T> read(const std::string& p, std::size_t n)
{
    std::vector<T> v(n);
    std::ifstream f(p, std::ios::binary);
    if (!f.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(sizeof(T) * n)))
        throw std::runtime_error("cannot read " + p);
    return v;
}

template <class T>
static void write(const std::string& p, const std::vector<T>& v)
{
    std::ofstream f(p, std::ios::binary);
    f.write(reinterpret_cast<const char*>(v.data()), static_cast<std::streamsize>(sizeof(T) * v.size()));
}

int main(int argc, char** argv)
{
    if (argc != 2)
    {
        std::cerr << "usage: host_engine_check <dir>\n";
        return 2;
    }
    const std::string d = argv[1];
    try
    {
        H::grid g;
        float eps, K, m, n, dt, U, D;
        {
            std::ifstream meta(d + "/meta.txt");
            meta >> g.n_rows >> g.n_cols >> g.cell_size >> g.boundary_conditions >> eps >> K >> m >> n >> dt >> U >> D;
            if (!meta) throw std::runtime_error("bad meta.txt");
        }
        const std::size_t cells = g.cells();
        const auto z = read<float>(d + "/z.f32", cells);
        const auto f = read<float>(d + "/f.f32", cells);
        const auto mask = read<std::uint8_t>(d + "/mask.u8", cells);
        const auto w = read<double>(d + "/w.f64", cells);

        write(d + "/filled.f32", H::fill_pits(g, z.data(), mask.data(), eps));

        H::flow_options o;
        o.allow_pits_as_outlets = true;
        H::flow_engine flow(g, f.data(), mask.data(), o);
        write(d + "/receiver.i64", flow.receivers());
        write(d + "/direction.u8", flow.directions());
        write(d + "/donors.u8", flow.donor_counts());
        write(d + "/outlets.i64", flow.outlets());
        write(d + "/topo.i64", flow.topological_order());
        write(d + "/svec.i64", flow.s_vector());
        write(d + "/start.i64", flow.s_vector_starts());
        write(d + "/size.u64", flow.s_vector_sizes());
        write(d + "/area.f64", flow.accumulate());
        write(d + "/weighted.f64", flow.accumulate(w));
        // per-cell queries against the bulk arrays
        std::vector<std::int64_t> ups;
        for (std::int64_t c = 0; c < static_cast<std::int64_t>(cells); c += 97)
        {
            if (!flow.is_valid_cell(c)) continue;
            if (flow.receiver_of(c) != flow.receivers()[c] || flow.donor_count_of(c) != flow.donor_counts()[c] ||
                flow.receiver_dir_of(c) != flow.directions()[c] || flow.is_outlet(c) != (flow.receivers()[c] == -2))
                throw std::runtime_error("per-cell query disagrees with the bulk arrays at " + std::to_string(c));
            const auto s = flow.upslope_nodes(c);
            ups.push_back(c);
            ups.push_back(static_cast<std::int64_t>(s.second));
            for (std::size_t i = 0; i < s.second; ++i)
            {
                ups.push_back(s.first[i]);
                if (!flow.is_upslope_of(s.first[i], c)) throw std::runtime_error("is_upslope_of disagrees");
            }
        }
        write(d + "/upslope.i64", ups);
        // two query rasters through the C++ layer
        {
            const auto q0 = flow.query(0);
            write(d + "/q_dist.f32", q0.data);
            write(d + "/q_dist_mask.u8", q0.mask);
            std::vector<float> vals(cells);
            for (std::size_t i = 0; i < cells; ++i) vals[i] = static_cast<float>(w[i]);
            const auto q7 = flow.query(7, vals, mask, {}, 1, true);
            write(d + "/q_upsum.f32", q7.data);
        }
        write(d + "/sp.f32", H::stream_power_d8(flow, f.data(), K, m, n, dt));

        lsdtt_gpu_lem_options lo{};
        lo.timestep = dt;
        lo.erodibility = K;
        lo.m_exponent = m;
        lo.n_exponent = n;
        lo.uplift_rate = U;
        lo.hillslope_diffusivity = D;
        lo.slope_clamp = 1e-5f;
        lo.fill_min_slope = 0.0f;
        lo.enable_hillslope = 1;
        lo.divide_area_by_dx = 1;
        lo.hillslope_rel_tol = 1e-8;
        lo.hillslope_max_iter = 2000;
        H::lem_engine lem(g, mask.data(), lo);
        std::vector<float> zl = f;
        const lsdtt_gpu_lem_stats st = lem.step(zl);
        write(d + "/lem.f32", zl);
        write(d + "/lem_stats.f32", std::vector<float>{st.delta_max_elevation, st.delta_mean_elevation,
                                                       st.max_local_elevation_change, st.mean_erosion_rate,
                                                       st.max_erosion_rate});

        // exception probes: the reference's exception types and messages
        std::ofstream errs(d + "/errors.txt");
        try { flow.receiver_of(-1); errs << "none\n"; }
        catch (const std::out_of_range& e) { errs << "out_of_range " << e.what() << "\n"; }
        try
        {
            H::flow_options strict;  // pits are not outlets: the unfilled surface has unresolved sinks
            H::flow_engine bad(g, z.data(), mask.data(), strict);
            errs << "none\n";
        }
        catch (const H::gb300_error& e) { errs << "runtime_error " << e.status() << " " << e.what() << "\n"; }
        try
        {
            H::flow_options forced;
            forced.allow_pits_as_outlets = true;
            forced.forced_outlet_flats = {static_cast<std::int64_t>(cells) + 5};
            H::flow_engine bad(g, f.data(), mask.data(), forced);
            errs << "none\n";
        }
        catch (const std::invalid_argument& e) { errs << "invalid_argument " << e.what() << "\n"; }
    }
    catch (const std::exception& e)
    {
        std::cerr << "host_engine_check: " << e.what() << "\n";
        return 1;
    }
    return 0;
}
