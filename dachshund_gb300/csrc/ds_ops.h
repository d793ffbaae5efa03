// Internal entry points shared between the translation units of the library.
#pragma once

#include <cstdio>
#include <new>

#include "ds_internal.cuh"

namespace ds {

// Runs f, mapping internal errors to status codes and the context's last
// error message (the C ABI's error convention).
template <class F>
int guarded(ds_context* ctx, F&& f) {
  // device buffers of this call are allocated / freed on the context's stream
  struct StreamScope {
    cudaStream_t prev;
    explicit StreamScope(cudaStream_t st) : prev(ds::g_alloc_stream) { ds::g_alloc_stream = st; }
    ~StreamScope() { ds::g_alloc_stream = prev; }
  } scope(ctx ? ctx->stream : nullptr);
  try {
    f();
    if (ctx) ctx->last_error.clear();
    return DS_OK;
  } catch (const Error& e) {
    if (ctx) ctx->last_error = e.msg;
    else fprintf(stderr, "[dachshund-gb300] %s\n", e.msg.c_str());
    return e.code;
  } catch (const std::bad_alloc&) {
    if (ctx) ctx->last_error = "host allocation failed";
    return DS_ERR_OOM;
  }
}

void gather_sorted(const PointSet& ps, const double* src, double* dst, cudaStream_t st);
void scatter_sorted(const PointSet& ps, const double* src, const double* scale, double* dst,
                    cudaStream_t st);
void vec_mul(int n, const double* a, const double* b, double* c, cudaStream_t st);

PairArgs op_pair_args(ds_operator* op, const double* v, double* out);
void op_apply_sorted(ds_operator* op, int epi, const double* v, double* out, cudaStream_t st);
void ensure_pcg_workspace(ds_operator* op);
void run_pcg(ds_operator* op, const ds_pcg_params& pp, ds_pcg_result& res, double* hist_out);

// Dense paths (dense.cu).
void op_build_dense(ds_operator* op);
void op_free_dense(ds_operator* op);
int dense_arith_in_use(const ds_operator* op);  // DS_DENSE_FLOAT_PAIR or DS_DENSE_FP64
// q = A v, with alpha = delta / (dotv . q) into *pcg when dotv is given, or
// r = b - A v (residual); returns at once when *skip != 0.
void dense_apply(ds_operator* op, bool residual, const double* v, double* out,
                 const double* dotv, PcgState* pcg, const int* skip, cudaStream_t st);
void solve_cf_dev(ds_context* ctx, int form, int n, const double* d_rec, const KernelConsts& kc,
                  const double* d_table, double* d_x);
// MapCovarDiag with the operator's table kernel: groups of map points as the
// right-hand sides of one multi-RHS FP64 PCG each (multi.cu).
void map_covar_diag_multi(ds_operator* op, int n_map, const double* map_pts,
                          const ds_pcg_params& pp, double* sigma_m, int* iters, int* success);

// The operator's tile-pair list, built on the first pair-kernel call
// (pcg.cu; op_pair_args calls it).
void ensure_op_pairs(ds_operator* op);

// The map's tiled point set, built on the first call that needs it (the
// structured column-grid map reads the points as given).
void ensure_map_points(ds_map* map);

// Mixed-precision form (mixed.cu).
void ensure_op_f32(ds_operator* op, double inner_cut);
void run_mixed(ds_operator* op, const ds_mixed_params& mp, ds_pcg_result& res,
               double* hist_out);
void map_product_f32_dev(ds_map* map, ds_operator* op, const double* x_dev, double* m_dev,
                         double cut);

}  // namespace ds
