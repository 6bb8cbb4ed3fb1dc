// ref_stubs.cpp -- test infrastructure only.
//
// The reference defines these two lsdtt_raster_meta members in
// src/core/lsdtt_raster_meta.cpp, which needs GDAL/OGR (absent here). Every
// raster the shim builds carries no CRS (empty crs_wkt). For such a raster the
// reference's check_projected_metres() finds neither a geographic CRS nor a
// non-metre unit and returns without effect (lsdtt_raster_meta.cpp:200-217),
// and the default synthetic georeference only sets CRS fields that nothing on
// the hot path reads. So both are no-ops here.

#include "lsdtt_raster_meta.hpp"

namespace lsdtt
{
void lsdtt_raster_meta::check_projected_metres() const {}
void lsdtt_raster_meta::set_default_synthetic_georeference() {}
} // namespace lsdtt
