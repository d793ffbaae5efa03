// Pixel record layouts (5 doubles) and map points (3 doubles), the binary
// formats of the reference (lib/pixel.h); the in-place casts between Pixel,
// NPixel and WPixel rely on the identical standard layout.
#ifndef DS_GB300_CXX_PIXEL_H
#define DS_GB300_CXX_PIXEL_H

struct Point { double x, y, z; };
struct Pixel { double x, y, z, n, d; };     // noise sigma n, data d
struct NPixel { double x, y, z, N, d; };    // N = n^2
struct WPixel { double x, y, z, w, wd; };   // w = 1/n, wd = d/n

Point* points_from_pixels_alloc(const int n, Pixel* const pixels);  // caller deletes[]
void pixel_to_npixel(const int n, Pixel* const p, NPixel* const np);
void npixel_to_pixel(const int n, NPixel* const np, Pixel* const p);
void pixel_to_wpixel(const int n, Pixel* const p, WPixel* const wp);
void wpixel_to_pixel(const int n, WPixel* const wp, Pixel* const p);

#endif
