// Structured form of the exact-kernel operator for skewers on a shared z grid
// (skewer_op.cu): the pixels are n_sk skewers of n_per records each (record
// s n_per + k is pixel k of skewer s), every skewer at its own (x, y) and all
// on the same z values z_0 < ... < z_{n_per - 1}, uniformly spaced.
#pragma once

#include "ds_internal.cuh"

namespace ds {

// Skewer pairs (a, b) within one cutoff, CSR by a (b ascending, a itself
// included): the perpendicular factor var_s exp(-c_perp |dxy_ab|^2) and the
// number of z levels kept, lev = 1 + max m with
// c_perp |dxy_ab|^2 + c_para (z_m - z_0)^2 < cut (built on the device).
struct SkewerNbrs {
  double cut = 0.0;
  int lmax = 0;        // largest L_ab
  long long n_terms = 0;  // sum over pairs of n_per (the apply kernel's FMAs)
  DevBuf<int> ptr, idx, lev;
  DevBuf<double> p64;
  DevBuf<float> p32;   // the factor in FP32 (inner lists)
};

struct SkewerGrid {
  int n_sk = 0, n_per = 0;
  double z0 = 0.0, dz = 0.0;  // the pixels' z grid: z_k = z0 + zd[k]
  DevBuf<double> taps64;  // exp(-c_para (z_m - z_0)^2), m < n_per
  SkewerNbrs outer;       // the operator's own cutoff (FP64-accurate residual)
  DevBuf<double> V64;     // (lmax + 1) x n: z-convolved column values per level
  // the FP32 inner operator of the mixed solve (its cutoff, built on demand)
  std::vector<double> zd;          // z_m - z_0
  DevBuf<double> sx, sy;           // skewer (x, y)
  SkewerNbrs inner;
  DevBuf<float> taps32, V32;
  DevBuf<double> dot_part;  // per-skewer p.q partials
  // record-order copies for the mixed solve (built on first use)
  DevBuf<double> rwl, rwr, re, rb, rx;
  DevBuf<float> rpd;
  // the persistent solve's CTA partials and barrier words (count, error code)
  DevBuf<double> p_part;
  DevBuf<int> p_sync;
  DevBuf<unsigned long long> p_time;  // its phase timers
  // float-pair copies for the persistent solve's FP64-accurate update
  // (record-order coefficients, outer factors, z taps; built on first use)
  DevBuf<float2> ff_wl, ff_wr, ff_e, ff_b, ff_op, ff_taps;
  // the persistent solve's product items (for the preconditioner and inner
  // cutoff they were built for)
  const void* res_pc = nullptr;
  double res_cut = 0.0;
  int res_max_list = 0;  // the most items of a block (above the limit: not built)
  DevBuf<int> it_cnt;            // per block: its items (n_blocks + 1: the largest)
  DevBuf<int> it_own;            // per block: its items on its own skewers (the first)
  DevBuf<unsigned int> it_off;   // item (slots of 512 per block): offset of its
                                 // (neighbour, level) row in the levels
  DevBuf<float4> it_coef;        // item: the factor for each of the block's skewers
};

// The vectors a structured product addresses: pos maps a record to its
// index in the vectors (null: the record's own index, the mixed solve's
// record order), wl, wr, e, b the operator's coefficients and right-hand side
// in that order.
struct SkewerVecs {
  const int* pos;
  const double *wl, *wr, *e, *b;
};
SkewerVecs skewer_vecs_sorted(ds_operator* op);
// record-order copies (built once; pdiag_sorted: the FP32 Jacobi diagonal)
SkewerVecs skewer_vecs_rec(ds_operator* op, const float* pdiag_sorted);
void skewer_x_to_rec(ds_operator* op, const double* x_sorted, double* x_rec, cudaStream_t st);
void skewer_x_to_sorted(ds_operator* op, const double* x_rec, double* x_sorted, cudaStream_t st);

// The FP32 inner product of the mixed solve, q = A32 p on FP32 vectors, with
// the PCG step's p.q and alpha = *num / p.q (written by the last CTA,
// counter reset to 0; counter null: no dot).  With beta non-null, p is first
// updated to z + beta p (the CG direction step).  ensure_skewer_inner builds
// the lists at the inner cutoff once.
void ensure_skewer_inner(ds_operator* op, double inner_cut);
void skewer_product_f32(ds_operator* op, const SkewerVecs& c, float* p, float* q,
                        unsigned int* counter, const double* num, double* alpha_out,
                        double* den_out, const int* skip, cudaStream_t st,
                        const double* beta = nullptr, const float* z = nullptr);

// r = b - A v (residual) or A v (product) with the structured FP64
// operator; the launch returns at once when *skip != 0 (skip may be null).
void skewer_apply_f64(ds_operator* op, const SkewerVecs& c, bool residual, const double* v,
                      double* out, const int* skip, cudaStream_t st);

// A map point set declared a grid of columns (ds_map_set_column_grid): point
// c nz + j at (X_c, Y_c, Z_j), the same Z_j in every column.  With an
// operator's skewer grid the map m = S_mp x becomes, per map column c and
// skewer b within the cutoff, P_cb times a z convolution of x_b sampled at
// the Z_j: the |Z_j - z_k| take Q distinct values (the two grids are
// commensurate), R_b^(q)[j] sums the pixels of the q nearest distance
// classes, and m[c, j] = sum_b P_cb R_b^(q_cb)[j] in FP64.
struct MapColumns {
  int ncol = 0, nz = 0;
  std::vector<double> z;   // Z_j
  DevBuf<double> cx, cy;   // column (x, y)
  // built for one operator and cutoff
  unsigned long long op_serial = 0;
  double cut = 0.0;
  int Q = 0, W = 0;                // distance classes, pixel window per Z_j
  DevBuf<int> kstart;              // first pixel index of Z_j's window
  DevBuf<signed char> cls;         // nz x W: distance class of each window pixel (-1: none)
  DevBuf<double> taps;             // Q: exp(-c_para delta_q^2)
  DevBuf<int> ptr, idx, lev;       // CSR column -> skewers, classes kept
  DevBuf<double> p64;              // var_s exp(-c_perp |dxy|^2)
  DevBuf<double> R;                // Q x n_sk x nz
  // the fused float-pair form (k_mc_fused): each column's list sorted by
  // classes kept (descending), its factor as a float pair, the class taps as
  // float pairs, and the operand split into float pairs per product
  DevBuf<int> fidx, flev;
  DevBuf<float2> fp, ftaps, xff;
};

struct OpF32;
struct SkewerPC;
// The structured mixed solve's iterations (band preconditioner whose blocks
// are whole skewers of the grid, record order) as one cooperative launch of
// CTAs that each own whole blocks and pass through the phases of each
// iteration between bounded grid barriers; r is the residual the start wrote
// (the recurrence updates it in place); false when the launch's conditions
// do not hold (nothing launched).  persistent_error reads (and
// clears) the error code of its barriers: 0, or the phase that timed out.
bool run_mixed_persistent(ds_operator* op, OpF32& f, const SkewerPC* pc, const SkewerVecs& sv,
                          double* X, float* r, int max_iter, cudaStream_t st);
int persistent_error(ds_operator* op, cudaStream_t st);
// The persistent launches' phase timers (ds_operator_get_persistent_profile):
// writes min(n, 26) values, returns that count (0: no launch yet).
int persistent_profile(ds_operator* op, double* out, int n, bool reset);

// m = S_mp x (caller order, device) with the structured FP64 map; false when
// the map or the operator has no grid (then nothing is launched).
bool skewer_map_product(ds_map* map, ds_operator* op, const double* x_dev, double* m_dev,
                        double cut);

}  // namespace ds
