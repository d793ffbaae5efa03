// Test driver: the Wiener-filter app path written against the library's C++
// interface (the reference's class and function names, dachshund_gb300/lib),
// i.e. read records -> W form -> GPU PCG -> map, plus the closed-form solve.
//
//   wf_app pixels.bin n lx ly lz nx ny nz tol max_iter step_r out_prefix
// writes out_prefix.map, out_prefix.x, out_prefix.xcf and prints
// "iters <n> success <0|1>".
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "dachshund.h"

static void write(const std::string& path, const double* v, int n) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f || fwrite(v, sizeof(double), n, f) != (size_t)n) exit(2);
  fclose(f);
}

int main(int argc, char** argv) {
  if (argc != 13) return 1;
  const int n = atoi(argv[2]);
  const double lx = atof(argv[3]), ly = atof(argv[4]), lz = atof(argv[5]);
  const int nx = atoi(argv[6]), ny = atoi(argv[7]), nz = atoi(argv[8]);
  const double tol = atof(argv[9]);
  const int max_iter = atoi(argv[10]), step_r = atoi(argv[11]);
  const std::string out = argv[12];
  const int n_map = nx * ny * nz;

  std::vector<Pixel> pixels(n);
  read_pixel_data(argv[1], n, pixels.data());
  std::vector<Point> map(n_map);
  init_uniform_map_coords(lx, ly, lz, nx, ny, nz, map.data());
  SignalCovarParams sp(0.0625, 2.5, 2.0);

  WPixel* wp = reinterpret_cast<WPixel*>(pixels.data());
  pixel_to_wpixel(n, pixels.data(), wp);
  std::vector<double> x(n, 0.0), xcf(n, 0.0), m(n_map);
  PCGResult r;
  {
    WFVectorW wf(n, wp, &sp);
    PCGParams pp = {n, max_iter, step_r, tol, false};
    r = wf.solve_pcg(pp, x.data());
    wf.solve_cf(xcf.data(), false, false);
  }
  Point* pc = points_from_pixels_alloc(n, pixels.data());
  smp_product(n, pc, n_map, map.data(), &sp, x.data(), m.data());
  delete[] pc;
  write(out + ".map", m.data(), n_map);
  write(out + ".x", x.data(), n);
  write(out + ".xcf", xcf.data(), n);
  printf("iters %d success %d\n", r.num_iters, r.success ? 1 : 0);
  return 0;
}
