/*
 * TEST INFRASTRUCTURE -- the CPU oracle for the Wiener-filter path.
 *
 * A plain-C (C11 + OpenMP) restatement of the reference's arithmetic for the
 * signal covariance, the two operator forms, Jacobi-PCG, the map product and
 * the map-covariance diagonals.  Only tests/, the smoke check and bench.py's
 * CPU-baseline leg may load it; the product never does.
 *
 * Records are arrays of 5 doubles per pixel, in the reference's struct
 * layouts (lib/pixel.h:16-50):
 *   Pixel  = {x, y, z, n, d}
 *   NPixel = {x, y, z, N = n*n, d}      (SN form)
 *   WPixel = {x, y, z, w = 1/n, wd = d/n} (W form)
 * Points are 3 doubles {x, y, z} (lib/pixel.h:8-12).
 *
 * Parity pins: oracle/_ref/libdsref.so (the unmodified reference compiled by
 * oracle/Makefile) and the golden vectors under tests/golden/.
 */
#ifndef DS_ORACLE_H
#define DS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define DSO_TABLE_N 200      /* default_gaussian_table_n, lib/signal_covar.h:8 */
#define DSO_TABLE_XMAX 4.0   /* default_gaussian_table_x_max, lib/signal_covar.h:7 */

typedef struct {
  double var_s;
  double c_perp;     /* 1 / (2 l_perp^2) */
  double c_para;     /* 1 / (2 l_para^2) */
  double dx_inv;     /* table index scale */
  double table[DSO_TABLE_N];
  int exact;         /* 0: table + linear interpolation; 1: exp() */
} dso_kernel;

void dso_kernel_init(dso_kernel* k, double var_s, double l_perp,
                     double l_para, int exact);
double dso_signal_covar(const dso_kernel* k, double perp2, double para2);

/* form: 0 = SN (NPixel records), 1 = W (WPixel records) */
void dso_A_product(const dso_kernel* k, int form, int n, const double* rec,
                   const double* a, double* b);
void dso_A_residual(const dso_kernel* k, int form, int n, const double* rec,
                    const double* x, double* r);
/* Rows [row0, row1) of A_product / smp_product: a bounded sample of the
 * same loops, for timing the CPU baseline on part of a large workload. */
void dso_A_product_rows(const dso_kernel* k, int form, int n, const double* rec,
                        const double* a, double* b, int row0, int row1);
void dso_smp_product_rows(const dso_kernel* k, int n_pix, const double* pix_pts,
                          const double* map_pts, const double* x, double* m,
                          int row0, int row1);
void dso_precond(const dso_kernel* k, int form, int n, const double* rec,
                 const double* r, double* s);
double dso_norm_b(int form, int n, const double* rec);

/* Jacobi-PCG; returns 1 on success.  hist receives up to max_hist norms. */
int dso_solve_pcg(const dso_kernel* k, int form, int n, const double* rec,
                  int max_iter, int step_r, double tol, double* x,
                  int* num_iters, double* hist, int max_hist, int* n_hist);

/* Dense closed-form solve via LDL^T (no pivoting; A is SPD). */
int dso_solve_cf(const dso_kernel* k, int form, int n, const double* rec,
                 double* x);

void dso_smp_product(const dso_kernel* k, int n_pix, const double* pix_pts,
                     int n_map, const double* map_pts, const double* x,
                     double* m);
void dso_sigma_m_noise_dom(const dso_kernel* k, int n_pix, const double* nrec,
                           int n_map, const double* map_pts, double* sigma_m);
void dso_map_covar_diag(const dso_kernel* k, int n_pix, const double* nrec,
                        int n_map, const double* map_pts, int max_iter,
                        int step_r, double tol, double* sigma_m, int* iters,
                        int* success);

void dso_init_uniform_map_coords(double lx, double ly, double lz, int nx,
                                 int ny, int nz, double* coords);
void dso_pixel_to_wpixel(int n, double* rec);
void dso_pixel_to_npixel(int n, double* rec);

#ifdef __cplusplus
}
#endif
#endif
