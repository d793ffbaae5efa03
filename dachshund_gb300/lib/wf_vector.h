// Wiener-filter operator classes with the reference's interface
// (lib/wf_vector.h): WFVectorSN, x = (S + N)^-1 d over NPixel records, and
// WFVectorW, x = w (w S w + I)^-1 w d over WPixel records.  Every method runs
// on the GPU through the C ABI (include/ds_gb300.h); the records are copied to
// the device on first use, so they must not change during the object's life
// (the reference holds them through a const pointer).
#ifndef DS_GB300_CXX_WF_VECTOR_H
#define DS_GB300_CXX_WF_VECTOR_H

#include <functional>

#include "pcg.h"
#include "pixel.h"
#include "signal_covar.h"

class WFVector {
 public:
  WFVector(const int num_pixels, const SignalCovarParams* const s_params)
      : n(num_pixels), s_params(s_params) {}
  const int n;
  const SignalCovarParams* const s_params;
};

// Shared GPU handle of an operator object (lazily created).
class WFVectorGpu {
 public:
  WFVectorGpu() : op_exact_(0), op_table_(0) {}
  ~WFVectorGpu();
  void* get(int form, int n, const double* records, const SignalCovarParams* p, bool exact);

 private:
  WFVectorGpu(const WFVectorGpu&);
  WFVectorGpu& operator=(const WFVectorGpu&);
  void* op_exact_;
  void* op_table_;
};

class WFVectorSN : public WFVector {
 public:
  const NPixel* const pixels;

  WFVectorSN(const int num_pixels, const NPixel* const pixels,
             const SignalCovarParams* const s_params);

  double A(const int i, const int j, const bool exact);
  double norm_b();
  void preconditioner_solve(const double* const b, double* const x);
  void A_product(const double* const a, double* const b);
  void A_residual(const double* const x, double* const r);

  std::function<void(const double* const, double* const)> this_pc_solve;
  std::function<void(const double* const, double* const)> this_A_product;
  std::function<void(const double* const, double* const)> this_A_residual;

  PCGResult solve_pcg(const PCGParams& pcg_params, double* const x);
  void solve_cf(double* const x, const bool verbose, const bool exact);

 private:
  WFVectorGpu gpu_;
};

class WFVectorW : public WFVector {
 public:
  const WPixel* const pixels;

  WFVectorW(const int num_pixels, const WPixel* const pixels,
            const SignalCovarParams* const s_params);

  double A(const int i, const int j, const bool exact);
  double norm_b();
  void preconditioner_solve(const double* const b, double* const x);
  void A_product(const double* const a, double* const b);
  void A_residual(const double* const x, double* const r);

  std::function<void(const double* const, double* const)> this_pc_solve;
  std::function<void(const double* const, double* const)> this_A_product;
  std::function<void(const double* const, double* const)> this_A_residual;

  PCGResult solve_pcg(const PCGParams& pcg_params, double* const x);
  void solve_cf(double* const x, const bool verbose, const bool exact);

 private:
  WFVectorGpu gpu_;
};

#endif
