// Record I/O and map-grid helpers with the reference's interface (lib/util.h).
#ifndef DS_GB300_CXX_UTIL_H
#define DS_GB300_CXX_UTIL_H

#include <string>

#include "map.h"

// Reads num_pixels Pixel records; exits with a message when the file cannot
// be opened or holds fewer records.
void read_pixel_data(const std::string path, const int num_pixels, Pixel* const pixels);

// Cell-centred uniform grid, flat index (ix * ny + iy) * nz + iz.
void init_uniform_map_coords(const double lx, const double ly, const double lz, const int nx,
                             const int ny, const int nz, Point* const coords);

void check_finite(const int n, const double* const v);

#endif
