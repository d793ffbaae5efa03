// Host-only driver of the C++ layer's record and map-grid helpers (no GPU
// call).  Usage: io_check <pixel file> <num_pixels> <nx> <ny> <nz>
//
// Reads the records with read_pixel_data (lib/util.cc:11-23 semantics, plus
// the record-count check), converts them to NPixel / WPixel and back in place
// (lib/pixel.cc:9-71), builds the uniform map grid (lib/util.cc:25-46) and
// prints everything with 17 significant digits for the Python side to compare.
#include <cstdio>
#include <cstdlib>

#include "dachshund.h"

static void print_pixels(const char* tag, const int n, const double* v) {
  for (int i = 0; i < n; ++i)
    printf("%s %.17g %.17g %.17g %.17g %.17g\n", tag, v[5 * i], v[5 * i + 1], v[5 * i + 2],
           v[5 * i + 3], v[5 * i + 4]);
}

int main(int argc, char** argv) {
  if (argc != 6) {
    fprintf(stderr, "usage: io_check <pixel file> <num_pixels> <nx> <ny> <nz>\n");
    return 2;
  }
  const int n = atoi(argv[2]);
  const int nx = atoi(argv[3]), ny = atoi(argv[4]), nz = atoi(argv[5]);
  Pixel* pixels = new Pixel[n];
  read_pixel_data(argv[1], n, pixels);
  print_pixels("P", n, &pixels[0].x);

  Point* pts = points_from_pixels_alloc(n, pixels);
  for (int i = 0; i < n; ++i) printf("Q %.17g %.17g %.17g\n", pts[i].x, pts[i].y, pts[i].z);
  delete[] pts;

  NPixel* np = reinterpret_cast<NPixel*>(pixels);
  pixel_to_npixel(n, pixels, np);
  print_pixels("N", n, &np[0].x);
  npixel_to_pixel(n, np, pixels);

  WPixel* wp = reinterpret_cast<WPixel*>(pixels);
  pixel_to_wpixel(n, pixels, wp);
  print_pixels("W", n, &wp[0].x);
  wpixel_to_pixel(n, wp, pixels);
  print_pixels("R", n, &pixels[0].x);
  delete[] pixels;

  Point* grid = new Point[(size_t)nx * ny * nz];
  init_uniform_map_coords(1.0 * nx, 2.0 * ny, 0.5 * nz, nx, ny, nz, grid);
  for (int i = 0; i < nx * ny * nz; ++i)
    printf("G %.17g %.17g %.17g\n", grid[i].x, grid[i].y, grid[i].z);
  delete[] grid;
  return 0;
}
