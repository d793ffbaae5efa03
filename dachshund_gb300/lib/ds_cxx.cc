// The reference's C++ library interface (lib/*.h) implemented over the C ABI
// of include/ds_gb300.h.  Host-side pieces (record conversions, the map grid,
// the timer, BLAS-1 helpers, file input) stay on the host as in the
// reference; every O(n^2) operation and every solve runs on the GPU.
// Errors follow the reference's convention: a message and exit(1) for
// unusable input or no GPU; PCGResult.success for solver outcomes.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "dachshund.h"
#include "ds_gb300.h"

// ---- GPU context (one per process) -----------------------------------------

static ds_context* gpu_context() {
  static ds_context* ctx = 0;
  if (!ctx) {
    const char* dev = getenv("DS_GB300_DEVICE");
    const int rc = ds_context_create(dev ? atoi(dev) : 0, &ctx);
    if (rc != DS_OK) {
      fprintf(stderr, "dachshund-gb300: no usable GPU (%s)\n", ds_status_string(rc));
      exit(1);
    }
  }
  return ctx;
}

static void check(int rc, const char* what) {
  if (rc == DS_OK) return;
  fprintf(stderr, "dachshund-gb300: %s failed: %s (%s)\n", what, ds_status_string(rc),
          ds_context_last_error(gpu_context()));
  exit(1);
}

static ds_kernel_params kernel_params(const SignalCovarParams* p, bool exact) {
  ds_kernel_params k;
  k.var_s = p->var_s;
  k.l_perp = p->l_perp();
  k.l_para = p->l_para();
  k.eval = exact ? DS_EVAL_EXACT : DS_EVAL_TABLE;
  k.exact_cutoff = 0.0;
  k.table = p->func_table;
  return k;
}

// ---- signal covariance ----------------------------------------------------

SignalCovarParams::SignalCovarParams(const double var_s, const double l_perp,
                                     const double l_para)
    : var_s(var_s), l_perp_(l_perp), l_para_(l_para) {
  gaussian_const_perp = 1.0 / (2.0 * l_perp * l_perp);
  gaussian_const_para = 1.0 / (2.0 * l_para * l_para);
  func_table_n = default_gaussian_table_n;
  func_table = new double[func_table_n];
  ds_table_init(func_table, &func_table_dx_inv);
}

SignalCovarParams::~SignalCovarParams() { delete[] func_table; }

// ---- records ----------------------------------------------------------------

Point* points_from_pixels_alloc(const int n, Pixel* const pixels) {
  Point* pts = new Point[n];
  for (int i = 0; i < n; ++i) {
    pts[i].x = pixels[i].x;
    pts[i].y = pixels[i].y;
    pts[i].z = pixels[i].z;
  }
  return pts;
}

void pixel_to_npixel(const int n, Pixel* const p, NPixel* const np) {
  for (int i = 0; i < n; ++i) {
    const Pixel q = p[i];
    np[i].x = q.x;
    np[i].y = q.y;
    np[i].z = q.z;
    np[i].N = q.n * q.n;
    np[i].d = q.d;
  }
}

void npixel_to_pixel(const int n, NPixel* const np, Pixel* const p) {
  for (int i = 0; i < n; ++i) {
    const NPixel q = np[i];
    p[i].x = q.x;
    p[i].y = q.y;
    p[i].z = q.z;
    p[i].n = sqrt(q.N);
    p[i].d = q.d;
  }
}

void pixel_to_wpixel(const int n, Pixel* const p, WPixel* const wp) {
  for (int i = 0; i < n; ++i) {
    const Pixel q = p[i];
    wp[i].x = q.x;
    wp[i].y = q.y;
    wp[i].z = q.z;
    wp[i].w = 1.0 / q.n;
    wp[i].wd = q.d / q.n;
  }
}

void wpixel_to_pixel(const int n, WPixel* const wp, Pixel* const p) {
  for (int i = 0; i < n; ++i) {
    const WPixel q = wp[i];
    p[i].x = q.x;
    p[i].y = q.y;
    p[i].z = q.z;
    p[i].n = 1.0 / q.w;
    p[i].d = q.wd / q.w;
  }
}

// ---- BLAS-1 -------------------------------------------------------------------

double ds_vector_dot(const int n, const double* const a, const double* const b) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

double ds_vector_norm(const int n, const double* const x) { return sqrt(ds_vector_dot(n, x, x)); }

void ds_vector_add_cv(const int n, const double a, const double* const b, double* const c) {
  for (int i = 0; i < n; ++i) c[i] += a * b[i];
}

void ds_vector_sub_cv(const int n, const double a, const double* const b, double* const c) {
  for (int i = 0; i < n; ++i) c[i] -= a * b[i];
}

// ---- timer ----------------------------------------------------------------------

Timer::Timer() { reset(); }
void Timer::reset() { t0 = get_time(); }
tv Timer::get_time() {
  tv t;
  gettimeofday(&t, NULL);
  return t;
}
double Timer::interval(const tv a, const tv b) {
  return (b.tv_sec - a.tv_sec) + 1.0e-6 * (b.tv_usec - a.tv_usec);
}
double Timer::elapsed() const { return interval(t0, get_time()); }
Timer total_timer;

// ---- input and the map grid ------------------------------------------------------

void read_pixel_data(const std::string path, const int num_pixels, Pixel* const pixels) {
  FILE* f = fopen(path.c_str(), "r");
  if (!f) {
    printf("Could not open file %s\n", path.c_str());
    exit(1);
  }
  const size_t got = fread(pixels, sizeof(Pixel), num_pixels, f);
  fclose(f);
  if (got != (size_t)num_pixels) {
    printf("File %s holds %zu pixel records, expected %d\n", path.c_str(), got, num_pixels);
    exit(1);
  }
}

void init_uniform_map_coords(const double lx, const double ly, const double lz, const int nx,
                             const int ny, const int nz, Point* const coords) {
  const double dx = lx / nx, dy = ly / ny, dz = lz / nz;
  for (int ix = 0; ix < nx; ++ix)
    for (int iy = 0; iy < ny; ++iy)
      for (int iz = 0; iz < nz; ++iz) {
        Point& p = coords[(ix * ny + iy) * nz + iz];
        p.x = dx * (ix + 0.5);
        p.y = dy * (iy + 0.5);
        p.z = dz * (iz + 0.5);
      }
}

void check_finite(const int n, const double* const v) {
  for (int i = 0; i < n; ++i)
    if (!std::isfinite(v[i])) printf("non-finite value v[%i] = %e\n", i, v[i]);
}

// ---- operators ---------------------------------------------------------------------

WFVectorGpu::~WFVectorGpu() {
  if (op_table_) ds_operator_destroy(static_cast<ds_operator*>(op_table_));
  if (op_exact_) ds_operator_destroy(static_cast<ds_operator*>(op_exact_));
}

void* WFVectorGpu::get(int form, int n, const double* records, const SignalCovarParams* p,
                       bool exact) {
  void*& slot = exact ? op_exact_ : op_table_;
  if (!slot) {
    const ds_kernel_params k = kernel_params(p, exact);
    ds_operator* op = 0;
    check(ds_operator_create(gpu_context(), form, n, records, &k, &op), "ds_operator_create");
    slot = op;
  }
  return slot;
}

template <class V>
static ds_operator* table_op(V* v, WFVectorGpu& gpu, int form) {
  return static_cast<ds_operator*>(
      gpu.get(form, v->n, reinterpret_cast<const double*>(v->pixels), v->s_params, false));
}

template <class V>
static double entry(V* v, WFVectorGpu& gpu, int form, int i, int j, bool exact) {
  double out = 0.0;
  check(ds_A_entries(table_op(v, gpu, form), exact ? DS_EVAL_EXACT : DS_EVAL_TABLE, 1, &i, &j,
                     &out),
        "ds_A_entries");
  return out;
}

template <class V>
static PCGResult solve(V* v, WFVectorGpu& gpu, int form, const PCGParams& pp, double* x) {
  ds_pcg_params p;
  p.max_iter = pp.max_iter;
  p.step_r = pp.step_r;
  p.tol = pp.tol;
  p.verbose = pp.verbose ? 1 : 0;
  std::vector<double> hist(pp.max_iter > 0 ? pp.max_iter + 1 : 2);
  ds_pcg_result r;
  const int rc = ds_solve_pcg(table_op(v, gpu, form), &p, x, &r, hist.data());
  if (rc != DS_OK && rc != DS_ERR_NOT_CONVERGED && rc != DS_ERR_NORM_B) check(rc, "ds_solve_pcg");
  PCGResult res;
  res.success = r.success != 0;
  res.num_iters = r.num_iters;
  if (rc != DS_ERR_NORM_B) res.residual_norms.assign(hist.begin(), hist.begin() + r.n_inner + 1);
  return res;
}

template <class V>
static void solve_closed_form(V* v, int form, double* x, bool verbose, bool exact) {
  if (verbose) puts("Solving the dense system on the GPU.");
  const ds_kernel_params k = kernel_params(v->s_params, exact);
  check(ds_solve_cf(gpu_context(), form, v->n, reinterpret_cast<const double*>(v->pixels), &k, x),
        "ds_solve_cf");
}

#define DS_WF_METHODS(CLASS, FORM, REC)                                                       \
  CLASS::CLASS(const int num_pixels, const REC* const pixels,                                \
               const SignalCovarParams* const s_params)                                      \
      : WFVector(num_pixels, s_params), pixels(pixels) {                                     \
    this_pc_solve = [this](const double* b, double* y) { preconditioner_solve(b, y); };     \
    this_A_product = [this](const double* a, double* b) { A_product(a, b); };               \
    this_A_residual = [this](const double* y, double* r) { A_residual(y, r); };             \
  }                                                                                          \
  double CLASS::A(const int i, const int j, const bool exact) {                              \
    return entry(this, gpu_, FORM, i, j, exact);                                             \
  }                                                                                          \
  double CLASS::norm_b() {                                                                   \
    double v = 0.0;                                                                          \
    check(ds_norm_b(table_op(this, gpu_, FORM), &v), "ds_norm_b");                          \
    return v;                                                                                \
  }                                                                                          \
  void CLASS::preconditioner_solve(const double* const b, double* const y) {                 \
    check(ds_preconditioner_solve(table_op(this, gpu_, FORM), b, y), "ds_preconditioner");   \
  }                                                                                          \
  void CLASS::A_product(const double* const a, double* const b) {                            \
    check(ds_A_product(table_op(this, gpu_, FORM), a, b), "ds_A_product");                   \
  }                                                                                          \
  void CLASS::A_residual(const double* const y, double* const r) {                           \
    check(ds_A_residual(table_op(this, gpu_, FORM), y, r), "ds_A_residual");                 \
  }                                                                                          \
  PCGResult CLASS::solve_pcg(const PCGParams& pp, double* const x) {                         \
    return solve(this, gpu_, FORM, pp, x);                                                   \
  }                                                                                          \
  void CLASS::solve_cf(double* const x, const bool verbose, const bool exact) {              \
    solve_closed_form(this, FORM, x, verbose, exact);                                        \
  }

DS_WF_METHODS(WFVectorSN, DS_FORM_SN, NPixel)
DS_WF_METHODS(WFVectorW, DS_FORM_W, WPixel)

// ---- map products -----------------------------------------------------------------

void smp_product(const int num_pixel_points, const Point* const pixel_coords,
                 const int num_map_points, const Point* const map_coords,
                 const SignalCovarParams* const s_params, const double* const x,
                 double* const m) {
  const ds_kernel_params k = kernel_params(s_params, false);
  check(ds_smp_product(gpu_context(), num_pixel_points,
                       reinterpret_cast<const double*>(pixel_coords), num_map_points,
                       reinterpret_cast<const double*>(map_coords), &k, x, m),
        "ds_smp_product");
}

void sigma_m_noise_dom(const int n_pix, const NPixel* pixels, const int n_map,
                       const Point* map_coords, const SignalCovarParams* s_params,
                       double* sigma_m) {
  const ds_kernel_params k = kernel_params(s_params, false);
  check(ds_sigma_m_noise_dom(gpu_context(), n_pix, reinterpret_cast<const double*>(pixels),
                             n_map, reinterpret_cast<const double*>(map_coords), &k, sigma_m),
        "ds_sigma_m_noise_dom");
}

PCGResult MapCovarDiag::solve_column_pcg(const int i, const PCGParams& pcg_params,
                                         double* const x) {
  // The column S_pm[:, i] as the right-hand side of an SN-form solve.
  std::vector<NPixel> col(pixels, pixels + n_pix);
  for (int k = 0; k < n_pix; ++k) {
    const double dx = map_coords[i].x - pixels[k].x, dy = map_coords[i].y - pixels[k].y;
    const double dz = map_coords[i].z - pixels[k].z;
    col[k].d = signal_covar(dx * dx + dy * dy, dz * dz, s_params);
  }
  WFVectorSN wf(n_pix, col.data(), s_params);
  return wf.solve_pcg(pcg_params, x);
}

std::vector<PCGResult> MapCovarDiag::solve_pcg(const PCGParams& pcg_params,
                                               double* const sigma_m) {
  std::vector<PCGResult> results(n_map);
  std::vector<int> iters(n_map), ok(n_map);
  const ds_kernel_params k = kernel_params(s_params, false);
  ds_pcg_params p;
  p.max_iter = pcg_params.max_iter;
  p.step_r = pcg_params.step_r;
  p.tol = pcg_params.tol;
  p.verbose = 0;
  check(ds_map_covar_diag(gpu_context(), n_pix, reinterpret_cast<const double*>(pixels), n_map,
                          reinterpret_cast<const double*>(map_coords), &k, &p, sigma_m,
                          iters.data(), ok.data()),
        "ds_map_covar_diag");
  for (int i = 0; i < n_map; ++i) {
    results[i].success = ok[i] != 0;
    results[i].num_iters = iters[i];
  }
  return results;
}
