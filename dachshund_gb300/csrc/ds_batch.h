// Batched solves over many independent chunks with several right-hand sides
// each: device layout, kernel arguments and the per-(chunk, RHS) CG state.
//
// Layout in HBM:
//   * each chunk is tiled on its own (k-d tiles of TILE pixels, padded per
//     chunk) and the chunks' tiles are concatenated: tile t belongs to chunk
//     tile_chunk[t], chunk c owns tiles [chunk_tile0[c], chunk_tile0[c + 1]);
//   * pixel coordinates (FP64 SoA and FP32 tile-relative) and coefficients
//     in that tile order; perm maps a sorted position to the caller's record
//     index (-1 on padding);
//   * every vector is pixel-major with the right-hand side fastest:
//     v[i * n_rhs + r], so one pixel's n_rhs values are contiguous;
//   * two culled tile-pair lists: the FP32 inner operator (inner cutoff) and
//     the FP64 residual operator (exact cutoff); no pair crosses a chunk.
#pragma once

#include "ds_f32.h"

namespace ds {

// Matvec variants the autotuner chooses from.
enum BatchVariant {
  BV_CUDA_CORE = 0,  // FP32 FMA/MUFU kernel, RB right-hand sides per pass
  BV_TENSOR = 1      // tcgen05 BF16 hi/lo S-tile x RHS contraction
};

struct BatchF32Args {
  const float4* xi;    // per pixel (tile-relative scaled coordinates, |xi|^2)
  const float4* orig;  // per tile
  const int* row_ptr;
  const int* cols;
  const unsigned short* mask;
  const int* row_order;
  int n_row_tiles;
  const int* tile_chunk;
  const int* chunk_done;
  const float* colw;
  const float* rowf;
  const float* ediag;
  int n_rhs;
  const float* p;  // [pixel][n_rhs]
  float* q;
  double* part;    // per (tile, RHS): p . q over the tile
  unsigned int* work;  // work-queue counter of the persistent launch
  unsigned long long* prof_pairs;  // profiling: pair x RHS products evaluated
  int formula;         // F32Formula of xi / rowf
  void* panel;         // tensor-core variant: BF16 hi / lo u panels
  int* err;            // tensor-core variant: error code of a timed-out wait
  long long wait_limit;  // tensor-core variant: bound of its waits (SM clock cycles)
};

struct BatchF64Args {
  KernelConsts kc;
  const double* x;
  const double* y;
  const double* z;
  const double* wl;
  const double* e;
  const double* b;   // [pixel][n_rhs]
  const double* xv;  // [pixel][n_rhs]
  double* r64;       // [pixel][n_rhs]
  float2* uu;        // [pixel][n_rhs]: var_s wl x as (hi, lo) floats
  FFPoints ff;       // float-pair coordinates (fx == nullptr: FP64 kernel value)
  const int* row_ptr;
  const int* cols;
  const unsigned short* mask;
  const int* row_order;
  int n_row_tiles;
  const int* tile_chunk;
  const int* chunk_done;
  const int* chunk_update;
  int n_rhs;
  unsigned int* work;
  unsigned long long* prof_pairs;  // profiling: pair x RHS products evaluated
};

// Per-(chunk, RHS) CG scalars (arrays of n_chunks * n_rhs, index c * R + r).
struct BatchState {
  int R;
  double tol;
  double delta;
  int max_iter;
  const int* chunk_tile0;
  double* rz;
  double* rz_old;
  double* alpha;
  double* beta;
  double* rmax;
  double* rbest;    // smallest recurrence |r| since the last halving
  double* rtrue;
  double* norm_b;
  double* tol_norm_b;
  int* iter;
  int* n_updates;
  int* need;
  int* hold;
  int* it_best;     // iteration of rbest
  int* stalled;     // the pending update was triggered by stagnation
  int* done;
  int* converged;
  int* chunk_done;
  int* chunk_update;
  int* active_chunks;
};

void launch_batch_mv_f32(const BatchF32Args& a, int formula, int rb, int grid, cudaStream_t st);
// Tensor-core variant (batch_tc.cu): RHS block 64, 32 or 16 (0: unsupported n_rhs).
int batch_tc_block(int R);
size_t batch_tc_panel_elems(int n_tiles, int R);
void launch_batch_mv_tc(const BatchF32Args& a, cudaStream_t st);
void launch_batch_resid_f64(const BatchF64Args& a, int grid, cudaStream_t st);

}  // namespace ds

struct ds_batch {
  ds_context* ctx = nullptr;
  int form = 0;
  int n_chunks = 0;
  int n_rhs = 0;
  int n_total = 0;   // pixels over all chunks
  int n_tiles = 0;
  int n_pad = 0;
  int formula = ds::F32_EXPANDED;
  double inner_cut = 24.0;
  ds::KernelConsts kc{};
  // chosen matvec variant (autotuner or caller)
  int variant = ds::BV_CUDA_CORE;
  int rb = 16;
  int grid_mv = 0;   // CTAs of the persistent matvec launch (0: one per row tile)
  bool tuned = false;
  ds::DevBuf<double> table;
  ds::DevBuf<double> x, y, z;
  ds::DevBuf<float4> xi, orig;
  ds::DevBuf<int> perm, tile_chunk, chunk_tile0;
  ds::PairList pairs32, pairs64;
  ds::DevBuf<double> wl, e, pdiag;
  ds::DevBuf<float> rowf, colw, ediag, pd32;
  ds::DevBuf<double> bv, xv, r64;
  ds::DevBuf<float2> uu;
  ds::FFData ffd;  // float-pair coordinates of the FP64-accurate residual
  ds::DevBuf<float> p, q, rr, zz, xc;
  ds::DevBuf<double> part;
  ds::DevBuf<double> s_rz, s_rz_old, s_alpha, s_beta, s_rmax, s_rbest, s_rtrue, s_norm_b,
      s_tol_norm_b;
  ds::DevBuf<int> s_iter, s_n_updates, s_need, s_hold, s_done, s_converged, s_it_best, s_stalled;
  ds::DevBuf<int> chunk_done, chunk_update, active;
  ds::DevBuf<int> loop_it;  // iterations run by the device-side loop of a solve
  ds::DevBuf<unsigned int> work;  // work-queue counters
  ds::DevBuf<unsigned short> panel;  // tensor-core variant: BF16 u panels (lazy)
  ds::DevBuf<int> err;               // tensor-core variant: time-out code
  ds::DevBuf<double> io_a, io_b;  // caller-order staging
  long long pairs32_total = 0;
  long long pairs64_total = 0;
  long long eval32 = 0;  // pairs in interacting sub-tile pairs, inner operator
  long long eval64 = 0;  // the same, FP64 residual operator
  int graph_replays = 0;
};

namespace ds {
bool batch_rb_supported(int R, int rb);
void batch_build(ds_batch* B, const double* d_rec, const int* sizes);
void batch_mv(ds_batch* B, cudaStream_t st);
void batch_resid(ds_batch* B, cudaStream_t st);
void batch_autotune(ds_batch* B, bool force, double* best_ms_out);
void batch_solve_dev(ds_batch* B, const ds_mixed_params& mp, const double* rhs_dev, double* x_dev,
                     int* iters, int* converged, int* n_updates, double* rel_resid,
                     double* seconds);
void batch_product_f32_dev(ds_batch* B, const double* p_dev, double* q_dev);
bool batch_variant_supported(const ds_batch* B, int variant);
}  // namespace ds
