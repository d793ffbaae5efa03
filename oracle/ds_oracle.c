/*
 * TEST INFRASTRUCTURE -- CPU oracle for the Wiener-filter path (see
 * ds_oracle.h).  Each function names the reference code it restates.  The
 * loops keep the reference's shape (OpenMP over rows, sequential inner sums
 * over j in input order, AoS records) so that, timed on the host cores, this
 * port also stands in for the reference's own CPU cost.
 */
#include "ds_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* SignalCovarParams ctor, lib/signal_covar.h:19-41: table f_i = exp(-i*dx)
 * on [0, x_max^2/2] with 200 knots. */
void dso_kernel_init(dso_kernel* k, double var_s, double l_perp,
                     double l_para, int exact) {
  k->var_s = var_s;
  k->c_perp = 1.0 / (2.0 * l_perp * l_perp);
  k->c_para = 1.0 / (2.0 * l_para * l_para);
  const double fx_max = DSO_TABLE_XMAX * DSO_TABLE_XMAX / 2.0;
  const double dx = fx_max / (DSO_TABLE_N - 1);
  k->dx_inv = 1.0 / dx;
  for (int i = 0; i < DSO_TABLE_N; ++i) k->table[i] = exp(-(dx * i));
  k->exact = exact;
}

/* linterp, lib/signal_covar.h:53-65: truncating index, zero past the
 * second-to-last knot. */
static inline double dso_linterp(const dso_kernel* k, double x) {
  const double xx = x * k->dx_inv;
  const int ix = (int)xx;
  if (ix > DSO_TABLE_N - 2) return 0.0;
  return k->table[ix] * (ix + 1 - xx) + k->table[ix + 1] * (xx - ix);
}

/* signal_covar / signal_covar_exact, lib/signal_covar.h:67-86. */
double dso_signal_covar(const dso_kernel* k, double perp2, double para2) {
  const double g = k->c_perp * perp2 + k->c_para * para2;
  if (k->exact) return k->var_s * exp(-g);
  return k->var_s * dso_linterp(k, g);
}

static inline double dso_pair_S(const dso_kernel* k, const double* pi,
                                const double* pj) {
  const double dx = pi[0] - pj[0];
  const double dy = pi[1] - pj[1];
  const double dz = pi[2] - pj[2];
  return dso_signal_covar(k, dx * dx + dy * dy, dz * dz);
}

/* Row i of A times v.
 * SN: A_ij = S_ij + N_i delta_ij          (lib/wf_vector.cc:16-40)
 * W:  A_ij = w_i S_ij w_j + delta_ij      (lib/wf_vector.cc:157-183) */
/* The evaluation mode and form are hoisted out of the j loop (the reference
 * compiles one loop per form with the table kernel inlined). */
#define DSO_ROW_LOOP(SEXPR, AEXPR)                          \
  for (int j = 0; j < n; ++j) {                             \
    const double* pj = rec + 5 * (size_t)j;                 \
    const double dx = pi[0] - pj[0];                        \
    const double dy = pi[1] - pj[1];                        \
    const double dz = pi[2] - pj[2];                        \
    const double perp2 = dx * dx + dy * dy;                 \
    const double para2 = dz * dz;                           \
    const double g = k->c_perp * perp2 + k->c_para * para2; \
    const double S = SEXPR;                                 \
    const double A = AEXPR;                                 \
    sum += A * v[j];                                        \
  }

static inline double dso_row_dot(const dso_kernel* k, int form, int n,
                                 const double* rec, int i, const double* v) {
  const double* pi = rec + 5 * (size_t)i;
  double sum = 0.0;
  if (k->exact) {
    if (form == 0) {
      DSO_ROW_LOOP(k->var_s * exp(-g), S + pi[3] * (i == j))
    } else {
      DSO_ROW_LOOP(k->var_s * exp(-g), pi[3] * S * pj[3] + (i == j))
    }
  } else {
    if (form == 0) {
      DSO_ROW_LOOP(k->var_s * dso_linterp(k, g), S + pi[3] * (i == j))
    } else {
      DSO_ROW_LOOP(k->var_s * dso_linterp(k, g), pi[3] * S * pj[3] + (i == j))
    }
  }
  return sum;
}

/* A_product, lib/wf_vector.cc:51-74 (SN) and :196-220 (W). */
void dso_A_product(const dso_kernel* k, int form, int n, const double* rec,
                   const double* a, double* b) {
  int i;
#pragma omp parallel for schedule(static)
  for (i = 0; i < n; ++i) b[i] = dso_row_dot(k, form, n, rec, i, a);
}

void dso_A_product_rows(const dso_kernel* k, int form, int n, const double* rec,
                        const double* a, double* b, int row0, int row1) {
  int i;
#pragma omp parallel for schedule(static)
  for (i = row0; i < row1; ++i) b[i - row0] = dso_row_dot(k, form, n, rec, i, a);
}

void dso_smp_product_rows(const dso_kernel* k, int n_pix, const double* pix_pts,
                          const double* map_pts, const double* x, double* m,
                          int row0, int row1) {
  int i;
#pragma omp parallel for schedule(static)
  for (i = row0; i < row1; ++i) {
    const double* mi = map_pts + 3 * (size_t)i;
    double sum = 0.0;
    for (int j = 0; j < n_pix; ++j)
      sum += dso_pair_S(k, mi, pix_pts + 3 * (size_t)j) * x[j];
    m[i - row0] = sum;
  }
}

/* A_residual, lib/wf_vector.cc:76-103 (SN) and :222-251 (W): r = b - A x
 * with b = d (SN) or wd (W), i.e. record field 4 in both layouts. */
void dso_A_residual(const dso_kernel* k, int form, int n, const double* rec,
                    const double* x, double* r) {
  int i;
#pragma omp parallel for schedule(static)
  for (i = 0; i < n; ++i)
    r[i] = rec[5 * (size_t)i + 4] - dso_row_dot(k, form, n, rec, i, x);
}

/* preconditioner_solve, lib/wf_vector.cc:42-49 (SN: 1/(var_s+N)) and
 * :185-194 (W: 1/(w^2 var_s + 1)). */
void dso_precond(const dso_kernel* k, int form, int n, const double* rec,
                 const double* r, double* s) {
  for (int i = 0; i < n; ++i) {
    const double f = rec[5 * (size_t)i + 3];
    const double diag = form == 0 ? k->var_s + f : f * f * k->var_s + 1.0;
    s[i] = r[i] / diag;
  }
}

/* norm_b, lib/wf_vector.cc:105-112 and :253-260. */
double dso_norm_b(int form, int n, const double* rec) {
  (void)form;
  double s = 0.0;
  for (int i = 0; i < n; ++i) {
    const double b = rec[5 * (size_t)i + 4];
    s += b * b;
  }
  return sqrt(s);
}

/* ds_vector_dot, lib/linalg.cc:9-17 (sequential sum). */
static double dso_dot(int n, const double* a, const double* b) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

/* pcg_solve + pcg_step, lib/pcg.h:27-160, followed by the W-form x *= w
 * (lib/wf_vector.cc:268-271). */
int dso_solve_pcg(const dso_kernel* k, int form, int n, const double* rec,
                  int max_iter, int step_r, double tol, double* x,
                  int* num_iters, double* hist, int max_hist, int* n_hist) {
  int nh = 0;
  const double norm_b = dso_norm_b(form, n, rec);
  *num_iters = 0;
  if (!(norm_b > 0.0)) {
    /* lib/pcg.h:79-86: early return, success = false. */
    *n_hist = 0;
    return 0;
  }
  double* d = (double*)malloc(sizeof(double) * n);
  double* r = (double*)malloc(sizeof(double) * n);
  double* s = (double*)malloc(sizeof(double) * n);
  double* q = (double*)malloc(sizeof(double) * n);
  const double tol_norm_b = tol * norm_b;

  dso_A_residual(k, form, n, rec, x, r);
  dso_precond(k, form, n, rec, r, d);
  double delta = dso_dot(n, r, d);
  double norm_r = sqrt(dso_dot(n, r, r));
  if (nh < max_hist) hist[nh++] = norm_r;

  int iter;
  for (iter = 1; iter < max_iter; ++iter) {
    const int full = (iter % step_r) == 0;
    dso_A_product(k, form, n, rec, d, q);
    const double alpha = delta / dso_dot(n, d, q);
    for (int i = 0; i < n; ++i) x[i] += alpha * d[i];
    if (full) {
      dso_A_residual(k, form, n, rec, x, r);
    } else {
      for (int i = 0; i < n; ++i) r[i] -= alpha * q[i];
    }
    dso_precond(k, form, n, rec, r, s);
    const double delta_old = delta;
    delta = dso_dot(n, r, s);
    const double beta = delta / delta_old;
    for (int i = 0; i < n; ++i) d[i] = s[i] + beta * d[i];
    norm_r = sqrt(dso_dot(n, r, r));
    if (nh < max_hist) hist[nh++] = norm_r;
    if (norm_r <= tol_norm_b) break;
  }
  free(d);
  free(r);
  free(s);
  free(q);
  if (form == 1)
    for (int i = 0; i < n; ++i) x[i] *= rec[5 * (size_t)i + 3];
  *num_iters = iter;
  *n_hist = nh;
  return iter == max_iter ? 0 : 1;
}

/* solve_cf, lib/wf_vector.cc:123-155 and :276-319: fill the dense A, then
 * solve.  The reference calls Eigen's pivoted LDL^T; A is SPD here, so an
 * unpivoted LDL^T gives the same solution to round-off. */
int dso_solve_cf(const dso_kernel* k, int form, int n, const double* rec,
                 double* x) {
  double* A = (double*)malloc(sizeof(double) * (size_t)n * n);
  double* D = (double*)malloc(sizeof(double) * n);
  if (!A || !D) {
    free(A);
    free(D);
    return 0;
  }
  int i;
#pragma omp parallel for schedule(static)
  for (i = 0; i < n; ++i) {
    const double* pi = rec + 5 * (size_t)i;
    for (int j = 0; j < n; ++j) {
      const double* pj = rec + 5 * (size_t)j;
      const double S = dso_pair_S(k, pi, pj);
      A[(size_t)i * n + j] =
          form == 0 ? S + pi[3] * (i == j) : pi[3] * S * pj[3] + (i == j);
    }
  }
  /* Right-looking LDL^T on the lower triangle: A = L D L^T, unit L. */
  int ok = 1;
  for (int j = 0; j < n; ++j) {
    const double djj = A[(size_t)j * n + j];
    if (!(djj > 0.0)) { ok = 0; break; }
    D[j] = djj;
    for (int r2 = j + 1; r2 < n; ++r2) A[(size_t)r2 * n + j] /= djj;
    int r2;
#pragma omp parallel for schedule(dynamic, 16)
    for (r2 = j + 1; r2 < n; ++r2) {
      const double f = A[(size_t)r2 * n + j] * djj;
      double* row = A + (size_t)r2 * n;
      for (int c = j + 1; c <= r2; ++c) row[c] -= f * A[(size_t)c * n + j];
    }
  }
  if (ok) {
    /* b = d (SN) or wd (W) */
    for (int r2 = 0; r2 < n; ++r2) x[r2] = rec[5 * (size_t)r2 + 4];
    for (int r2 = 0; r2 < n; ++r2) {          /* L y = b */
      double s = x[r2];
      for (int c = 0; c < r2; ++c) s -= A[(size_t)r2 * n + c] * x[c];
      x[r2] = s;
    }
    for (int r2 = 0; r2 < n; ++r2) x[r2] /= D[r2];
    for (int r2 = n - 1; r2 >= 0; --r2) {     /* L^T x = y */
      double s = x[r2];
      for (int c = r2 + 1; c < n; ++c) s -= A[(size_t)c * n + r2] * x[c];
      x[r2] = s;
    }
    if (form == 1)
      for (int r2 = 0; r2 < n; ++r2) x[r2] *= rec[5 * (size_t)r2 + 3];
  }
  free(A);
  free(D);
  return ok;
}

/* smp_product, lib/map.cc:20-43. */
void dso_smp_product(const dso_kernel* k, int n_pix, const double* pix_pts,
                     int n_map, const double* map_pts, const double* x,
                     double* m) {
  int i;
#pragma omp parallel for schedule(static)
  for (i = 0; i < n_map; ++i) {
    const double* mi = map_pts + 3 * (size_t)i;
    double sum = 0.0;
    for (int j = 0; j < n_pix; ++j)
      sum += dso_pair_S(k, mi, pix_pts + 3 * (size_t)j) * x[j];
    m[i] = sum;
  }
}

/* sigma_m_noise_dom, lib/map_covar.cc:11-38: sum_j S_ij^2 / N_j. */
void dso_sigma_m_noise_dom(const dso_kernel* k, int n_pix, const double* nrec,
                           int n_map, const double* map_pts, double* sigma_m) {
  int i;
#pragma omp parallel for schedule(static)
  for (i = 0; i < n_map; ++i) {
    const double* mi = map_pts + 3 * (size_t)i;
    double sum = 0.0;
    for (int j = 0; j < n_pix; ++j) {
      const double* pj = nrec + 5 * (size_t)j;
      const double S = dso_pair_S(k, mi, pj);
      const double W = 1.0 / pj[3];
      sum += S * W * S;
    }
    sigma_m[i] = sum;
  }
}

/* MapCovarDiag::solve_column_pcg + solve_pcg, lib/map_covar.cc:40-113: for
 * each map point, solve (S+N) x = S_pm[:, i] by SN-form PCG from x = 0, then
 * sigma_m[i] = S_mp[i, :] . x when the solve succeeded. */
void dso_map_covar_diag(const dso_kernel* k, int n_pix, const double* nrec,
                        int n_map, const double* map_pts, int max_iter,
                        int step_r, double tol, double* sigma_m, int* iters,
                        int* success) {
  double* col = (double*)malloc(sizeof(double) * 5 * (size_t)n_pix);
  double* x = (double*)malloc(sizeof(double) * n_pix);
  double* srow = (double*)malloc(sizeof(double) * n_pix);
  double hist[1];
  int nh;
  memcpy(col, nrec, sizeof(double) * 5 * (size_t)n_pix);
  for (int i = 0; i < n_map; ++i) {
    const double* mi = map_pts + 3 * (size_t)i;
    for (int j = 0; j < n_pix; ++j) {
      srow[j] = dso_pair_S(k, mi, nrec + 5 * (size_t)j);
      col[5 * (size_t)j + 4] = srow[j];
      x[j] = 0.0;
    }
    int it = 0;
    const int ok = dso_solve_pcg(k, 0, n_pix, col, max_iter, step_r, tol, x,
                                 &it, hist, 0, &nh);
    double s = 0.0;
    if (ok)
      for (int j = 0; j < n_pix; ++j) s += srow[j] * x[j];
    sigma_m[i] = s;
    iters[i] = it;
    success[i] = ok;
  }
  free(col);
  free(x);
  free(srow);
}

/* init_uniform_map_coords, lib/util.cc:25-46: cell centres, flat index
 * (ix*ny + iy)*nz + iz (z fastest). */
void dso_init_uniform_map_coords(double lx, double ly, double lz, int nx,
                                 int ny, int nz, double* coords) {
  const double dx = lx / nx, dy = ly / ny, dz = lz / nz;
  for (int ix = 0; ix < nx; ++ix)
    for (int iy = 0; iy < ny; ++iy)
      for (int iz = 0; iz < nz; ++iz) {
        const size_t i = ((size_t)ix * ny + iy) * nz + iz;
        coords[3 * i + 0] = dx * (ix + 0.5);
        coords[3 * i + 1] = dy * (iy + 0.5);
        coords[3 * i + 2] = dz * (iz + 0.5);
      }
}

/* pixel_to_wpixel / pixel_to_npixel, lib/pixel.cc:23-58 (in place). */
void dso_pixel_to_wpixel(int n, double* rec) {
  for (int i = 0; i < n; ++i) {
    double* p = rec + 5 * (size_t)i;
    const double ni = p[3];
    p[3] = 1.0 / ni;
    p[4] = p[4] / ni;
  }
}

void dso_pixel_to_npixel(int n, double* rec) {
  for (int i = 0; i < n; ++i) {
    double* p = rec + 5 * (size_t)i;
    p[3] = p[3] * p[3];
  }
}
