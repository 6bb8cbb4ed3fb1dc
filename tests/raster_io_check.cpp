// Command-line driver of lsdtt_gb300/host/raster_io.hpp for
// tests/test_raster_io.py:
//   read  <raster> <out-prefix>   -> <out-prefix>.data (float32), .mask (uint8), .meta (text)
//   write <values.f32> <rows> <cols> <x_min> <y_min> <cell> <nodata> <envi|esri> <raster> [wkt]
// Exit code 3 with the message on stderr when the library throws.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "lsdtt_gb300/host/raster_io.hpp"

int main(int argc, char** argv)
{
    try
    {
        const std::string mode = argc > 1 ? argv[1] : "";
        if (mode == "read" && argc == 4)
        {
            const lsdtt_gb300::raster_grid g = lsdtt_gb300::read_raster(argv[2]);
            const std::string pre = argv[3];
            std::ofstream(pre + ".data", std::ios::binary)
                .write(reinterpret_cast<const char*>(g.data.data()), static_cast<std::streamsize>(g.data.size() * 4));
            std::ofstream(pre + ".mask", std::ios::binary)
                .write(reinterpret_cast<const char*>(g.mask.data()), static_cast<std::streamsize>(g.mask.size()));
            std::ofstream m(pre + ".meta");
            m.precision(17);
            m << g.meta.n_rows << " " << g.meta.n_cols << " " << g.meta.x_min << " " << g.meta.y_min << " "
              << g.meta.cell_size << " " << g.meta.no_data_value << "\n"
              << g.meta.crs_wkt << "\n";
            return 0;
        }
        if (mode == "write" && (argc == 11 || argc == 12))
        {
            lsdtt_gb300::raster_meta meta;
            meta.n_rows = std::atoi(argv[3]);
            meta.n_cols = std::atoi(argv[4]);
            meta.x_min = std::atof(argv[5]);
            meta.y_min = std::atof(argv[6]);
            meta.cell_size = std::atof(argv[7]);
            meta.no_data_value = std::atof(argv[8]);
            if (argc == 12) meta.crs_wkt = argv[11];
            std::vector<float> v(static_cast<std::size_t>(meta.n_rows) * meta.n_cols);
            std::ifstream f(argv[2], std::ios::binary);
            f.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(v.size() * 4));
            const std::string fmt = argv[9];
            lsdtt_gb300::write_raster(argv[10], v, meta,
                                      fmt == "esri" ? lsdtt_gb300::raster_format::esri_gridfloat
                                                    : lsdtt_gb300::raster_format::envi_bil);
            return 0;
        }
        std::cerr << "usage: read <raster> <prefix> | write <values> <rows> <cols> <x_min> <y_min> <cell> <nodata> "
                     "<envi|esri> <raster> [wkt]\n";
        return 2;
    }
    catch (const std::exception& e)
    {
        std::cerr << e.what() << "\n";
        return 3;
    }
}
