// PCG parameter/result types and the generic host PCG driver with the
// reference's interface (lib/pcg.h).  The WFVector classes of this library do
// not use the host driver: their solve_pcg runs the whole iteration on the
// GPU (ds_solve_pcg).  pcg_solve stays for callers that drive their own
// operator through std::function callbacks.
#ifndef DS_GB300_CXX_PCG_H
#define DS_GB300_CXX_PCG_H

#include <cmath>
#include <cstdio>
#include <functional>
#include <vector>

#include "linalg.h"

struct PCGParams {
  int n;
  int max_iter;
  int step_r;   // full residual b - A x every step_r iterations
  double tol;   // stop when |r| <= tol |b|
  bool verbose;
};

struct PCGResult {
  bool success;
  int num_iters;
  std::vector<double> residual_norms;
};

typedef std::function<void(const double*, double*)> ds_apply_fn;

// One CG step: q = A d; x += alpha d; r -= alpha q (or r = b - A x on full
// steps); s = M^-1 r; d = s + beta d.
static inline void pcg_step(const int n, ds_apply_fn A_product, ds_apply_fn A_residual,
                            ds_apply_fn preconditioner_solve, double* const d,
                            double* const q, double* const r, double* const s,
                            double* const x, const bool full_residual,
                            double* const delta) {
  A_product(d, q);
  const double alpha = *delta / ds_vector_dot(n, d, q);
  ds_vector_add_cv(n, alpha, d, x);
  if (full_residual)
    A_residual(x, r);
  else
    ds_vector_sub_cv(n, alpha, q, r);
  preconditioner_solve(r, s);
  const double delta_old = *delta;
  *delta = ds_vector_dot(n, r, s);
  const double beta = *delta / delta_old;
  for (int i = 0; i < n; ++i) d[i] = s[i] + beta * d[i];
}

static inline PCGResult pcg_solve(const PCGParams& params, const double norm_b,
                                  ds_apply_fn A_product, ds_apply_fn A_residual,
                                  ds_apply_fn preconditioner_solve, double* const x) {
  const int n = params.n;
  PCGResult res;
  res.success = false;
  res.num_iters = 0;
  if (norm_b <= 0.0) {
    puts("[WARNING] Requested PCG solve where |b| <= 0.0. Returning early.\n");
    return res;
  }
  std::vector<double> d(n), r(n), s(n), q(n);
  const double tol_norm_b = params.tol * norm_b;
  A_residual(x, r.data());
  preconditioner_solve(r.data(), d.data());
  double delta = ds_vector_dot(n, r.data(), d.data());
  double norm_r = ds_vector_norm(n, r.data());
  res.residual_norms.push_back(norm_r);
  if (params.verbose) {
    printf("[PCG] Solving %i x %i problem.\n", n, n);
    printf("    Goal |r| < (tol) |b| = %e,  delta = %e\n", tol_norm_b, delta);
  }
  int iter;
  for (iter = 1; iter < params.max_iter; ++iter) {
    pcg_step(n, A_product, A_residual, preconditioner_solve, d.data(), q.data(), r.data(),
             s.data(), x, iter % params.step_r == 0, &delta);
    norm_r = ds_vector_norm(n, r.data());
    res.residual_norms.push_back(norm_r);
    if (norm_r <= tol_norm_b) {
      if (params.verbose)
        printf("    iter %i reached |r| = %e < tol |b| = %e\n", iter, norm_r, tol_norm_b);
      break;
    }
    if (params.verbose) printf("    iter %i, |r| %e, delta %e\n", iter, norm_r, delta);
  }
  res.success = iter < params.max_iter;
  if (!res.success) puts("[WARNING] PCG reached max iteration before stop condition.");
  res.num_iters = iter;
  return res;
}

#endif
