// Test infrastructure: a C-callable harness over the UNMODIFIED reference
// library (caseywstark/dachshund lib/*.cc), compiled from the reference's own
// sources by oracle/Makefile into oracle/_ref/libdsref.so.  It exists only so
// that the tests and the oracle restatement can be checked against what the
// reference itself computes; nothing in the product links or loads it.
//
// Every entry point takes plain arrays of 5-double pixel records, laid out as
// the reference's Pixel/NPixel/WPixel structs (lib/pixel.h:16-50), and calls
// the reference function named in its comment.

#include <cstring>
#include <vector>

#include "dachshund.h"

extern "C" {

// SignalCovarParams ctor table (lib/signal_covar.h:19-41).
void dsref_table(double var_s, double l_perp, double l_para, double* table,
                 double* dx_inv, double* c_perp, double* c_para) {
  SignalCovarParams p(var_s, l_perp, l_para);
  std::memcpy(table, p.func_table, sizeof(double) * p.func_table_n);
  *dx_inv = p.func_table_dx_inv;
  *c_perp = p.gaussian_const_perp;
  *c_para = p.gaussian_const_para;
}

// signal_covar / signal_covar_exact (lib/signal_covar.h:67-86), elementwise.
void dsref_signal_covar(double var_s, double l_perp, double l_para, int n,
                        const double* perp2, const double* para2, int exact,
                        double* out) {
  SignalCovarParams p(var_s, l_perp, l_para);
  for (int i = 0; i < n; ++i)
    out[i] = exact ? signal_covar_exact(perp2[i], para2[i], &p)
                   : signal_covar(perp2[i], para2[i], &p);
}

// form 0 = SN (NPixel records), form 1 = W (WPixel records).
// WFVector{SN,W}::A_product (lib/wf_vector.cc:51-74, 196-220).
void dsref_A_product(int form, int n, const double* rec, double var_s,
                     double l_perp, double l_para, const double* a,
                     double* b) {
  SignalCovarParams p(var_s, l_perp, l_para);
  if (form == 0) {
    WFVectorSN v(n, reinterpret_cast<const NPixel*>(rec), &p);
    v.A_product(a, b);
  } else {
    WFVectorW v(n, reinterpret_cast<const WPixel*>(rec), &p);
    v.A_product(a, b);
  }
}

// WFVector{SN,W}::A_residual (lib/wf_vector.cc:76-103, 222-251).
void dsref_A_residual(int form, int n, const double* rec, double var_s,
                      double l_perp, double l_para, const double* x,
                      double* r) {
  SignalCovarParams p(var_s, l_perp, l_para);
  if (form == 0) {
    WFVectorSN v(n, reinterpret_cast<const NPixel*>(rec), &p);
    v.A_residual(x, r);
  } else {
    WFVectorW v(n, reinterpret_cast<const WPixel*>(rec), &p);
    v.A_residual(x, r);
  }
}

// WFVector{SN,W}::A(i, j, exact) (lib/wf_vector.cc:16-40, 157-183), for a
// list of (i, j) index pairs.
void dsref_A_entries(int form, int n, const double* rec, double var_s,
                     double l_perp, double l_para, int exact, int m,
                     const int* ii, const int* jj, double* out) {
  SignalCovarParams p(var_s, l_perp, l_para);
  if (form == 0) {
    WFVectorSN v(n, reinterpret_cast<const NPixel*>(rec), &p);
    for (int k = 0; k < m; ++k) out[k] = v.A(ii[k], jj[k], exact != 0);
  } else {
    WFVectorW v(n, reinterpret_cast<const WPixel*>(rec), &p);
    for (int k = 0; k < m; ++k) out[k] = v.A(ii[k], jj[k], exact != 0);
  }
}

// WFVector{SN,W}::solve_pcg (lib/wf_vector.cc:114-121, 263-274) driving
// pcg_solve (lib/pcg.h:67-160).  x is the initial guess on input and the
// solution on output.  Returns success; writes num_iters and up to
// max_hist residual norms (the count is returned in *n_hist).
int dsref_solve_pcg(int form, int n, const double* rec, double var_s,
                    double l_perp, double l_para, int max_iter, int step_r,
                    double tol, double* x, int* num_iters, double* hist,
                    int max_hist, int* n_hist) {
  SignalCovarParams p(var_s, l_perp, l_para);
  PCGParams pp = {n, max_iter, step_r, tol, false};
  PCGResult res;
  if (form == 0) {
    WFVectorSN v(n, reinterpret_cast<const NPixel*>(rec), &p);
    res = v.solve_pcg(pp, x);
  } else {
    WFVectorW v(n, reinterpret_cast<const WPixel*>(rec), &p);
    res = v.solve_pcg(pp, x);
  }
  *num_iters = res.success || !res.residual_norms.empty() ? res.num_iters : 0;
  int k = 0;
  for (; k < (int)res.residual_norms.size() && k < max_hist; ++k)
    hist[k] = res.residual_norms[k];
  *n_hist = k;
  return res.success ? 1 : 0;
}

// WFVector{SN,W}::solve_cf (lib/wf_vector.cc:123-155, 276-319).
void dsref_solve_cf(int form, int n, const double* rec, double var_s,
                    double l_perp, double l_para, int exact, double* x) {
  SignalCovarParams p(var_s, l_perp, l_para);
  if (form == 0) {
    WFVectorSN v(n, reinterpret_cast<const NPixel*>(rec), &p);
    v.solve_cf(x, false, exact != 0);
  } else {
    WFVectorW v(n, reinterpret_cast<const WPixel*>(rec), &p);
    v.solve_cf(x, false, exact != 0);
  }
}

// smp_product (lib/map.cc:20-43).  Points are 3-double records (lib/pixel.h:8-12).
void dsref_smp_product(int n_pix, const double* pix_pts, int n_map,
                       const double* map_pts, double var_s, double l_perp,
                       double l_para, const double* x, double* m) {
  SignalCovarParams p(var_s, l_perp, l_para);
  smp_product(n_pix, reinterpret_cast<const Point*>(pix_pts), n_map,
              reinterpret_cast<const Point*>(map_pts), &p, x, m);
}

// sigma_m_noise_dom (lib/map_covar.cc:11-38), NPixel records.
void dsref_sigma_m_noise_dom(int n_pix, const double* nrec, int n_map,
                             const double* map_pts, double var_s,
                             double l_perp, double l_para, double* sigma_m) {
  SignalCovarParams p(var_s, l_perp, l_para);
  sigma_m_noise_dom(n_pix, reinterpret_cast<const NPixel*>(nrec), n_map,
                    reinterpret_cast<const Point*>(map_pts), &p, sigma_m);
}

// MapCovarDiag::solve_pcg (lib/map_covar.cc:73-113), NPixel records.
// Writes per-map-point iteration counts and success flags.
void dsref_map_covar_diag(int n_pix, const double* nrec, int n_map,
                          const double* map_pts, double var_s, double l_perp,
                          double l_para, int max_iter, int step_r, double tol,
                          double* sigma_m, int* iters, int* success) {
  SignalCovarParams p(var_s, l_perp, l_para);
  PCGParams pp = {n_pix, max_iter, step_r, tol, false};
  MapCovarDiag mcd(n_pix, reinterpret_cast<const NPixel*>(nrec), n_map,
                   reinterpret_cast<const Point*>(map_pts), &p);
  std::vector<PCGResult> res = mcd.solve_pcg(pp, sigma_m);
  for (int i = 0; i < n_map && i < (int)res.size(); ++i) {
    iters[i] = res[i].num_iters;
    success[i] = res[i].success ? 1 : 0;
  }
}

// init_uniform_map_coords (lib/util.cc:25-46).
void dsref_init_uniform_map_coords(double lx, double ly, double lz, int nx,
                                   int ny, int nz, double* coords) {
  init_uniform_map_coords(lx, ly, lz, nx, ny, nz,
                          reinterpret_cast<Point*>(coords));
}

// pixel_to_wpixel / pixel_to_npixel (lib/pixel.cc:23-58), in place.
void dsref_pixel_to_wpixel(int n, double* rec) {
  pixel_to_wpixel(n, reinterpret_cast<Pixel*>(rec),
                  reinterpret_cast<WPixel*>(rec));
}
void dsref_pixel_to_npixel(int n, double* rec) {
  pixel_to_npixel(n, reinterpret_cast<Pixel*>(rec),
                  reinterpret_cast<NPixel*>(rec));
}

}  // extern "C"
