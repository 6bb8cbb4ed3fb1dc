// raster_io.hpp -- GDAL-free raster input and output for the GPU path's
// callers: ENVI rasters (.bil / .bsq / .img with an ENVI .hdr) and ESRI
// GridFloat (.flt with its .hdr), read into and written from row-major
// float32 arrays with the metadata the GPU entry points take.
//
// The reference does all raster I/O through GDAL (lsdtt_data_loader,
// src/core/lsdtt_data_loader.hpp:395-560), which is absent here; this header
// covers the two plain binary formats a DEM pipeline exchanges without it and
// keeps the reference's conventions:
//   * rows run north to south (the first row of the array is the top row);
//   * the metadata mirror lsdtt_raster_meta (src/core/lsdtt_raster_meta.hpp):
//     x_min / y_min the left and bottom edges, square cells (non-square
//     pixels are refused, as the reference's loader refuses them),
//     no_data_value, the CRS as WKT where the header carries one;
//   * a pixel equal to no_data_value or not finite is nodata: its mask is 0
//     and its value becomes no_data_value (read_tile, lsdtt_data_loader.cpp
//     :725-745), so mask == 0 always means "data holds no_data_value".
// Header-only; host code, no CUDA.
#pragma once

#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace lsdtt_gb300
{

struct raster_meta
{
    int n_rows = 0;
    int n_cols = 0;
    double x_min = 0.0;      // left edge
    double y_min = 0.0;      // bottom edge
    double cell_size = 1.0;  // square cells
    double no_data_value = -9999.0;
    std::string crs_wkt;     // empty: none
};

struct raster_grid
{
    std::vector<float> data;          // n_rows x n_cols, top row first
    std::vector<std::uint8_t> mask;   // 1 valid, 0 nodata
    raster_meta meta;
};

enum class raster_format
{
    envi_bil,      // ENVI header + one band of float32, little endian
    esri_gridfloat // ESRI .hdr (ncols/nrows/xllcorner/...) + .flt float32
};

namespace raster_io_detail
{

inline std::string lower(std::string s)
{
    for (char& c : s) c = static_cast<char>(std::tolower(static_cast<unsigned char>(c)));
    return s;
}

inline std::string trim(const std::string& s)
{
    const auto a = s.find_first_not_of(" \t\r\n");
    if (a == std::string::npos) return std::string();
    const auto b = s.find_last_not_of(" \t\r\n");
    return s.substr(a, b - a + 1);
}

// The header that goes with a data file: name.hdr, else name.ext.hdr.
inline std::string header_path(const std::string& data_path)
{
    const auto dot = data_path.find_last_of('.');
    const auto slash = data_path.find_last_of("/\\");
    std::string a = (dot != std::string::npos && (slash == std::string::npos || dot > slash))
                        ? data_path.substr(0, dot) + ".hdr"
                        : data_path + ".hdr";
    std::ifstream fa(a);
    if (fa.good()) return a;
    return data_path + ".hdr";
}

inline bool host_little_endian()
{
    const std::uint16_t one = 1;
    unsigned char b[2];
    std::memcpy(b, &one, 2);
    return b[0] == 1;
}

inline void swap_bytes(unsigned char* p, std::size_t width, std::size_t count)
{
    for (std::size_t i = 0; i < count; ++i)
        for (std::size_t k = 0; k < width / 2; ++k) std::swap(p[i * width + k], p[i * width + width - 1 - k]);
}

// Values of one band in file order, converted to float.
inline std::vector<float> read_samples(const std::string& path, std::size_t offset, std::size_t count, int envi_type,
                                       bool little)
{
    std::size_t width = 0;
    switch (envi_type)
    {
    case 1: width = 1; break;   // uint8
    case 2: width = 2; break;   // int16
    case 3: width = 4; break;   // int32
    case 4: width = 4; break;   // float32
    case 5: width = 8; break;   // float64
    case 12: width = 2; break;  // uint16
    case 13: width = 4; break;  // uint32
    default: throw std::runtime_error("raster_io: unsupported ENVI data type " + std::to_string(envi_type));
    }
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("raster_io: cannot open " + path);
    f.seekg(static_cast<std::streamoff>(offset));
    std::vector<unsigned char> raw(width * count);
    f.read(reinterpret_cast<char*>(raw.data()), static_cast<std::streamsize>(raw.size()));
    if (static_cast<std::size_t>(f.gcount()) != raw.size())
        throw std::runtime_error("raster_io: " + path + " is shorter than its header says");
    if (width > 1 && little != host_little_endian()) swap_bytes(raw.data(), width, count);
    std::vector<float> out(count);
    const unsigned char* p = raw.data();
    for (std::size_t i = 0; i < count; ++i, p += width)
    {
        switch (envi_type)
        {
        case 1: out[i] = static_cast<float>(*p); break;
        case 2: { std::int16_t v; std::memcpy(&v, p, 2); out[i] = static_cast<float>(v); break; }
        case 3: { std::int32_t v; std::memcpy(&v, p, 4); out[i] = static_cast<float>(v); break; }
        case 4: { float v; std::memcpy(&v, p, 4); out[i] = v; break; }
        case 5: { double v; std::memcpy(&v, p, 8); out[i] = static_cast<float>(v); break; }
        case 12: { std::uint16_t v; std::memcpy(&v, p, 2); out[i] = static_cast<float>(v); break; }
        default: { std::uint32_t v; std::memcpy(&v, p, 4); out[i] = static_cast<float>(v); break; }
        }
    }
    return out;
}

// The nodata rule of the reference's loader: equal to the sentinel or not
// finite -> mask 0 and the sentinel as the value.
inline void apply_nodata(raster_grid& g)
{
    const float nd = static_cast<float>(g.meta.no_data_value);
    g.mask.assign(g.data.size(), 1);
    for (std::size_t i = 0; i < g.data.size(); ++i)
    {
        const float v = g.data[i];
        if (v == nd || !std::isfinite(v))
        {
            g.mask[i] = 0;
            g.data[i] = nd;
        }
    }
}

// "{a, b, c}" -> fields (braces of the value removed, split at top-level commas)
inline std::vector<std::string> brace_fields(const std::string& v)
{
    std::string s = trim(v);
    if (!s.empty() && s.front() == '{') s = s.substr(1);
    if (!s.empty() && s.back() == '}') s.pop_back();
    std::vector<std::string> out;
    int depth = 0;
    std::string cur;
    for (char c : s)
    {
        if (c == '{' || c == '[') ++depth;
        if (c == '}' || c == ']') --depth;
        if (c == ',' && depth == 0)
        {
            out.push_back(trim(cur));
            cur.clear();
        }
        else
            cur += c;
    }
    if (!trim(cur).empty()) out.push_back(trim(cur));
    return out;
}

inline void check_square(double dx, double dy, const std::string& path)
{
    if (!(dx > 0.0) || !(dy > 0.0) || std::fabs(dx - dy) > 1e-9 * std::fmax(dx, dy))
        throw std::runtime_error("raster_io: " + path + " has non-square or invalid pixels (" + std::to_string(dx) +
                                 " x " + std::to_string(dy) + "); square cells are required");
}

inline raster_grid read_envi(const std::string& data_path, const std::string& hdr_text)
{
    // key = value, values in braces may span lines
    std::vector<std::pair<std::string, std::string>> kv;
    {
        std::istringstream in(hdr_text);
        std::string line, pending_key, pending_val;
        int depth = 0;
        std::getline(in, line);  // "ENVI"
        while (std::getline(in, line))
        {
            if (depth > 0)
            {
                pending_val += "\n" + line;
            }
            else
            {
                const auto eq = line.find('=');
                if (eq == std::string::npos) continue;
                pending_key = lower(trim(line.substr(0, eq)));
                pending_val = line.substr(eq + 1);
            }
            depth = 0;
            for (char c : pending_val)
            {
                if (c == '{') ++depth;
                if (c == '}') --depth;
            }
            if (depth <= 0)
            {
                kv.emplace_back(pending_key, trim(pending_val));
                depth = 0;
            }
        }
    }
    auto get = [&](const std::string& k) -> const std::string* {
        for (const auto& p : kv)
            if (p.first == k) return &p.second;
        return nullptr;
    };
    auto need_int = [&](const std::string& k) {
        const std::string* v = get(k);
        if (!v) throw std::runtime_error("raster_io: ENVI header of " + data_path + " has no '" + k + "'");
        return std::stoi(*v);
    };
    raster_grid g;
    g.meta.n_cols = need_int("samples");
    g.meta.n_rows = need_int("lines");
    const int bands = get("bands") ? std::stoi(*get("bands")) : 1;
    if (bands != 1)
        throw std::runtime_error("raster_io: " + data_path + " has " + std::to_string(bands) +
                                 " bands; one is supported");
    const std::size_t offset = get("header offset") ? static_cast<std::size_t>(std::stoll(*get("header offset"))) : 0;
    const int type = need_int("data type");
    const bool little = !(get("byte order") && std::stoi(*get("byte order")) == 1);
    if (const std::string* di = get("data ignore value")) g.meta.no_data_value = std::stod(*di);
    if (const std::string* cs = get("coordinate system string"))
    {
        std::string w = trim(*cs);
        if (!w.empty() && w.front() == '{') w = w.substr(1);
        if (!w.empty() && w.back() == '}') w.pop_back();
        g.meta.crs_wkt = trim(w);
    }
    double dx = 1.0, dy = 1.0, ex = 0.0, ny = 0.0, rx = 1.0, ry = 1.0;
    if (const std::string* mi = get("map info"))
    {
        const auto f = brace_fields(*mi);
        if (f.size() < 7) throw std::runtime_error("raster_io: malformed 'map info' in the header of " + data_path);
        rx = std::stod(f[1]);
        ry = std::stod(f[2]);
        ex = std::stod(f[3]);
        ny = std::stod(f[4]);
        dx = std::stod(f[5]);
        dy = std::stod(f[6]);
    }
    check_square(dx, dy, data_path);
    // the reference pixel (1-based, at its upper-left corner) -> edges
    g.meta.cell_size = dx;
    g.meta.x_min = ex - (rx - 1.0) * dx;
    const double y_max = ny + (ry - 1.0) * dy;
    g.meta.y_min = y_max - g.meta.n_rows * dy;
    const std::size_t n = static_cast<std::size_t>(g.meta.n_rows) * static_cast<std::size_t>(g.meta.n_cols);
    g.data = read_samples(data_path, offset, n, type, little);
    apply_nodata(g);
    return g;
}

inline raster_grid read_gridfloat(const std::string& data_path, const std::string& hdr_text)
{
    raster_grid g;
    bool centre_x = false, centre_y = false, have_x = false, have_y = false, little = true;
    double xll = 0.0, yll = 0.0;
    std::istringstream in(hdr_text);
    std::string line;
    while (std::getline(in, line))
    {
        std::istringstream ls(line);
        std::string k, v;
        if (!(ls >> k >> v)) continue;
        k = lower(k);
        if (k == "ncols") g.meta.n_cols = std::stoi(v);
        else if (k == "nrows") g.meta.n_rows = std::stoi(v);
        else if (k == "xllcorner" || k == "xllcenter")
        {
            xll = std::stod(v);
            centre_x = k == "xllcenter";
            have_x = true;
        }
        else if (k == "yllcorner" || k == "yllcenter")
        {
            yll = std::stod(v);
            centre_y = k == "yllcenter";
            have_y = true;
        }
        else if (k == "cellsize") g.meta.cell_size = std::stod(v);
        else if (k == "nodata_value") g.meta.no_data_value = std::stod(v);
        else if (k == "byteorder") little = lower(v) != "msbfirst";
    }
    if (g.meta.n_rows <= 0 || g.meta.n_cols <= 0 || !have_x || !have_y)
        throw std::runtime_error("raster_io: the header of " + data_path + " lacks ncols, nrows or the corner");
    check_square(g.meta.cell_size, g.meta.cell_size, data_path);
    g.meta.x_min = centre_x ? xll - 0.5 * g.meta.cell_size : xll;
    g.meta.y_min = centre_y ? yll - 0.5 * g.meta.cell_size : yll;
    const std::size_t n = static_cast<std::size_t>(g.meta.n_rows) * static_cast<std::size_t>(g.meta.n_cols);
    g.data = read_samples(data_path, 0, n, 4, little);
    apply_nodata(g);
    return g;
}

inline void write_floats(const std::string& path, const std::vector<float>& data)
{
    std::ofstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("raster_io: cannot write " + path);
    if (host_little_endian())
        f.write(reinterpret_cast<const char*>(data.data()), static_cast<std::streamsize>(data.size() * 4));
    else
    {
        std::vector<float> c(data);
        swap_bytes(reinterpret_cast<unsigned char*>(c.data()), 4, c.size());
        f.write(reinterpret_cast<const char*>(c.data()), static_cast<std::streamsize>(c.size() * 4));
    }
    if (!f) throw std::runtime_error("raster_io: writing " + path + " failed");
}

inline std::string fmt_double(double v)
{
    std::ostringstream o;
    o.precision(17);
    o << v;
    return o.str();
}

}  // namespace raster_io_detail

// Read a raster: ENVI (the header's first line is "ENVI") or ESRI GridFloat.
inline raster_grid read_raster(const std::string& data_path)
{
    using namespace raster_io_detail;
    const std::string hp = header_path(data_path);
    std::ifstream hf(hp);
    if (!hf) throw std::runtime_error("raster_io: no header for " + data_path + " (looked for " + hp + ")");
    std::stringstream ss;
    ss << hf.rdbuf();
    const std::string text = ss.str();
    if (lower(trim(text.substr(0, text.find('\n')))) == "envi") return read_envi(data_path, text);
    return read_gridfloat(data_path, text);
}

// Write a raster as float32 with its header next to it (name.hdr).
// `data` is n_rows x n_cols, top row first.
inline void write_raster(const std::string& data_path, const std::vector<float>& data, const raster_meta& meta,
                         raster_format fmt = raster_format::envi_bil)
{
    using namespace raster_io_detail;
    if (!(meta.n_rows > 0 && meta.n_cols > 0 && meta.cell_size > 0.0))
        throw std::runtime_error("raster_io: invalid raster metadata");
    if (data.size() != static_cast<std::size_t>(meta.n_rows) * static_cast<std::size_t>(meta.n_cols))
        throw std::runtime_error("raster_io: " + std::to_string(data.size()) + " values for a " +
                                 std::to_string(meta.n_rows) + " x " + std::to_string(meta.n_cols) + " raster");
    const auto dot = data_path.find_last_of('.');
    const auto slash = data_path.find_last_of("/\\");
    const std::string hp = (dot != std::string::npos && (slash == std::string::npos || dot > slash))
                               ? data_path.substr(0, dot) + ".hdr"
                               : data_path + ".hdr";
    std::ofstream h(hp);
    if (!h) throw std::runtime_error("raster_io: cannot write " + hp);
    if (fmt == raster_format::envi_bil)
    {
        const double y_max = meta.y_min + meta.n_rows * meta.cell_size;
        h << "ENVI\n"
          << "samples = " << meta.n_cols << "\n"
          << "lines = " << meta.n_rows << "\n"
          << "bands = 1\n"
          << "header offset = 0\n"
          << "data type = 4\n"
          << "interleave = bil\n"
          << "byte order = 0\n"
          << "map info = {Arbitrary, 1, 1, " << fmt_double(meta.x_min) << ", " << fmt_double(y_max) << ", "
          << fmt_double(meta.cell_size) << ", " << fmt_double(meta.cell_size) << "}\n"
          << "data ignore value = " << fmt_double(meta.no_data_value) << "\n";
        if (!meta.crs_wkt.empty()) h << "coordinate system string = {" << meta.crs_wkt << "}\n";
    }
    else
    {
        h << "ncols " << meta.n_cols << "\n"
          << "nrows " << meta.n_rows << "\n"
          << "xllcorner " << fmt_double(meta.x_min) << "\n"
          << "yllcorner " << fmt_double(meta.y_min) << "\n"
          << "cellsize " << fmt_double(meta.cell_size) << "\n"
          << "NODATA_value " << fmt_double(meta.no_data_value) << "\n"
          << "byteorder LSBFIRST\n";
    }
    if (!h) throw std::runtime_error("raster_io: writing " + hp + " failed");
    write_floats(data_path, data);
}

}  // namespace lsdtt_gb300
