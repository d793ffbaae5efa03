// Signal covariance parameters and the scalar kernel, with the interface of
// the reference's lib/signal_covar.h (same class, members and functions) so
// that its callers build unchanged.  The GPU kernels evaluate the same
// arithmetic (include/ds_gb300.h, DS_EVAL_TABLE / DS_EVAL_EXACT).
#ifndef DS_GB300_CXX_SIGNAL_COVAR_H
#define DS_GB300_CXX_SIGNAL_COVAR_H

#include <cmath>

const double default_gaussian_table_x_max = 4.0;  // table spans exponents [0, x_max^2 / 2]
const int default_gaussian_table_n = 200;         // knots

class SignalCovarParams {
 public:
  double var_s;
  double gaussian_const_perp;  // 1 / (2 l_perp^2)
  double gaussian_const_para;  // 1 / (2 l_para^2)
  int func_table_n;
  double func_table_dx_inv;
  double* func_table;          // f_i = exp(-i dx), i < func_table_n

  SignalCovarParams(const double var_s, const double l_perp, const double l_para);
  ~SignalCovarParams();

  // The correlation lengths as given (the GPU layer passes these, not the
  // derived constants, so both sides compute identical constants).
  double l_perp() const { return l_perp_; }
  double l_para() const { return l_para_; }

 private:
  double l_perp_, l_para_;
  SignalCovarParams(const SignalCovarParams&);             // owns func_table
  SignalCovarParams& operator=(const SignalCovarParams&);
};

// Linear interpolation of the table at x >= 0; 0 once the truncated index
// passes the second-to-last knot.
static inline double linterp(const double x, const int n, const double dx_inv,
                             const double* const f) {
  const double xx = x * dx_inv;
  const int ix = (int)xx;
  if (ix > n - 2) return 0.0;
  return f[ix] * (ix + 1 - xx) + f[ix + 1] * (xx - ix);
}

static inline double signal_covar(const double x_perp_2, const double x_para_2,
                                  const SignalCovarParams* const p) {
  const double g = p->gaussian_const_perp * x_perp_2 + p->gaussian_const_para * x_para_2;
  return p->var_s * linterp(g, p->func_table_n, p->func_table_dx_inv, p->func_table);
}

static inline double signal_covar_exact(const double x_perp_2, const double x_para_2,
                                        const SignalCovarParams* const p) {
  const double g = p->gaussian_const_perp * x_perp_2 + p->gaussian_const_para * x_para_2;
  return p->var_s * exp(-g);
}

#endif
