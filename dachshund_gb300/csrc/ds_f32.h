// FP32 side of the mixed-precision form: tile-relative scaled coordinates,
// the FP32 pair-kernel arguments and the reliable-update PCG state.
#pragma once

#include <memory>

#include "ds_internal.cuh"

namespace ds {

enum F32Formula { F32_EXPANDED = 0, F32_DIRECT = 1 };

// Tile-relative FP32 coordinates of a PointSet, scaled so that
// |dX|^2 = (c_perp dperp^2 + c_para dz^2) log2(e).
struct F32Points {
  DevBuf<float4> orig;  // per tile: origin (x, y, z, 0)
  DevBuf<float4> xi;    // per point: (xi_x, xi_y, xi_z, |xi|^2)
  double max_a = 0.0;   // max |xi|^2 (bounds 2^|xi|^2 of the EXPANDED formula)
};

void build_f32_points(F32Points& fp, const PointSet& ps, double sx, double sy, double sz,
                      cudaStream_t st);

struct F32Args {
  const float4* rxi; const float4* rorig;
  const float4* cxi; const float4* corig;
  const int* row_ptr; const int* cols;
  int n_row_tiles;
  const unsigned short* mask;  // sub-tile interaction mask per tile pair
  const int* item_ptr;         // work items per row tile (PairList::items)
  const unsigned int* items;
  const int* row_order;        // blockIdx -> row tile (heaviest first), or null
  const float* colw;   // column weights (W: w_j, SN: 1)
  const float* v;      // column vector
  // EPI_PRODUCT
  const float* rowf;   // wl_i var_s 2^-|xi_i|^2 (EXPANDED) or wl_i var_s (DIRECT)
  const float* ediag;  // diagonal e_i
  const float* vrow;   // row-side vector of the diagonal term
  float* out;
  const float* dotv;   // fused FP64 dot dotv . out -> *den_out, *alpha_out = *num / dot
  double* dot_partial;
  unsigned int* counter;
  const double* num;
  double* alpha_out;
  double* den_out;
  const int* skip_flag;
  // EPI_MAP
  const int* row_perm;
  double* out64;
  // profiling
  long long n_tile_pairs;
  unsigned long long* prof_pairs;
  Profiler* prof;
  int* err;        // tensor-core kernel: error code of a timed-out wait (device)
  float* tc_cols;  // tensor-core kernel: column operands (n_row_tiles x 2048 floats)
};

void launch_pair_f32(int formula, int epi, const F32Args& a, cudaStream_t st);

// The inner product q = A32 p with the pair exponents on the tensor cores
// (pair_tc.cu): EXPANDED formula, EPI_PRODUCT epilogue, a.err set.
bool pair_tc_usable(int formula, int epi, const F32Args& a);
void launch_pair_tc(const F32Args& a, cudaStream_t st);

// Inner-matvec kernel of the mixed-precision form (ds_operator_set_inner_matvec).
enum InnerVariant { INNER_AUTO = 0, INNER_CUDA_CORE = 1, INNER_TENSOR = 2, INNER_STRUCTURED = 3 };

// Float-pair coordinates for the FP64-accurate residual on the FP32 pipe
// (pair_ff.cu): per pixel its coordinates scaled by sqrt(c_perp),
// sqrt(c_para) relative to its tile's (scaled) origin; per tile the origin.
struct FFPoints {
  const float2* fx;
  const float2* fy;
  const float2* fz;
  const double* orig;  // 3 per tile
  double sp, sq;       // sqrt(c_perp), sqrt(c_para)
};

struct FFData {
  DevBuf<float2> fx, fy, fz;
  DevBuf<double> orig;
  FFPoints view{};
};

bool ff_usable(const KernelConsts& kc);
void build_ff_points(FFData& f, const PointSet& ps, const KernelConsts& kc, cudaStream_t st);
void launch_pair_ff_resid(const KernelConsts& kc, const PairArgs& a, const FFPoints& f,
                          cudaStream_t st);

// Device state of the reliable-update mixed-precision PCG.
struct MixedState {
  double rz;          // r . z (FP32 vectors, FP64 sum)
  double rz_old;
  double alpha;
  double beta;
  double pq;
  double rnorm;       // |r| of the FP32 recurrence
  double rmax;        // largest |r| since the last reliable update
  double rtrue;       // last FP64 true-residual norm
  double norm_b;
  double tol_norm_b;
  double delta;       // reliable-update trigger: |r| < delta * rmax
  double rbest;       // smallest |r| since the last halving (stagnation test)
  int it_best;        // iteration of rbest
  int stalled;        // the pending update was triggered by stagnation
  int iter;           // FP32 iterations done
  int max_iter;
  int done;
  int converged;
  int need_update;    // a reliable update is due this iteration
  int skip_update;    // == !need_update (skip flag of the update kernels)
  int n_updates;      // FP64 residual evaluations
  int pad;
  int init_skip;      // skip the FP64-accurate initial residual (x0 = 0, or the
                      // FP32 one is far above tol)
  int pad2;
  unsigned int counter[4];
};

// FP32 operator data, built on the first mixed-precision call.
struct OpF32 {
  double inner_cut = 0.0;
  int formula = F32_EXPANDED;
  F32Points pts;
  PairList pairs;                   // at inner_cut (built on first use: ensure_f32_pairs)
  bool pairs_built = false;
  DevBuf<float> rowf, colw, ediag, pdiag;
  DevBuf<float> p, q, r, z;         // FP32 iteration vectors (sorted, padded)
  DevBuf<float> r2;                 // second r buffer of the band preconditioner
  DevBuf<MixedState> state;
  HostBuf<MixedState> h_state;      // pinned staging of the state
  DevBuf<double> hist, htrue;
  bool use_ff = false;  // outer residual in float-float arithmetic (else FP64)
  FFData ffd;
  DevBuf<int> tc_err;     // error flag of the tensor-core inner matvec
  DevBuf<float> tc_cols;  // its column operands (16 floats per point)
};

// FP32 data of a map point set (DIRECT formula only).
struct MapF32 {
  unsigned long long op_serial = 0;
  double cut = 0.0;
  F32Points pts;
  PairList pairs;
  DevBuf<float> rowf;
  DevBuf<float> xs;  // FP32 copy of the solution, sorted
};

}  // namespace ds
