// Device helpers shared by the kernels: deterministic block reductions, the
// "last block finishes" pattern, and the FP64 signal-covariance evaluations.
#pragma once

#include <cuda_runtime.h>

#include "ds_internal.cuh"

namespace ds {

// Sum of v over the block; valid in thread 0.  Fixed order (shuffle tree
// within warps, then warps in order), so results are run-to-run identical.
template <int NT>
__device__ __forceinline__ double block_sum(double v, double* sm /* NT/32 */) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();  // sm may still be read by a previous call
  if (lane == 0) sm[wid] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < NT / 32; ++w) s += sm[w];
  return s;
}

// Every block calls this once after writing its partial result (thread 0);
// returns true in exactly one block, the last to arrive, which then sees all
// partials.  The counter is reset by that block.
__device__ __forceinline__ bool last_block_arrive(unsigned int* counter) {
  __shared__ bool am_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned int prev = atomicAdd(counter, 1u);
    am_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (am_last) __threadfence();
  return am_last;
}

// Deterministic sum of n partials (stride `stride`, offset `off`) by one block.
template <int NT>
__device__ __forceinline__ double reduce_partials(const double* part, int n, int stride, int off,
                                                  double* sm) {
  double v = 0.0;
  for (int k = threadIdx.x; k < n; k += NT) v += __ldcg(part + (size_t)k * stride + off);
  return block_sum<NT>(v, sm);
}

// Table kernel in the reference's exact operation order
// (lib/signal_covar.h:53-77, argument as in lib/wf_vector.cc:162-167):
// products and sums rounded separately, truncating index, zero once the
// index passes the second-to-last knot.  Same-skewer pixels 8 Mpc/h apart
// land exactly on xx = 199.0 with l_para = 2, so the argument must round
// exactly like the reference for the cutoff to agree.
__device__ __forceinline__ double s_table_f64(double dx, double dy, double dz,
                                              const KernelConsts& k, const double* tf) {
  const double perp2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
  const double para2 = __dmul_rn(dz, dz);
  const double g = __dadd_rn(__dmul_rn(k.c_perp, perp2), __dmul_rn(k.c_para, para2));
  const double xx = __dmul_rn(g, k.dx_inv);
  const bool inside = xx < (double)(TABLE_N - 1);
  int ix = __double2int_rz(xx);
  ix = min(max(ix, 0), TABLE_N - 2);
  const double lo = __dsub_rn((double)(ix + 1), xx);
  const double hi = __dsub_rn(xx, (double)ix);
  const double gp = __dadd_rn(__dmul_rn(tf[ix], lo), __dmul_rn(tf[ix + 1], hi));
  return inside ? __dmul_rn(k.var_s, gp) : 0.0;
}

// Table kernel without var_s (folded into the column weights): the argument
// and the interpolation weights are bit-identical to the reference's
// (lib/signal_covar.h:53-65); the truncating index comes from a round-down
// add of 1.5 * 2^52 instead of a double->int conversion (slower than an FP64
// FMA on GB300): for 0 <= xx < 2^51, t = xx + 1.5*2^52 rounded down holds
// floor(xx) in its low mantissa bits and t - 1.5*2^52 == floor(xx) exactly.
__device__ __forceinline__ double gp_table_fast(double dx, double dy, double dz,
                                                const KernelConsts& k, const double* tf) {
  const double perp2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
  const double para2 = __dmul_rn(dz, dz);
  const double g = __dadd_rn(__dmul_rn(k.c_perp, perp2), __dmul_rn(k.c_para, para2));
  const double xx = __dmul_rn(g, k.dx_inv);
  const double M = 6755399441055744.0;
  const double t = __dadd_rd(xx, M);
  const double fl = t - M;
  const int ix = min(max(__double2loint(t), 0), TABLE_N - 2);
  const double lo = (fl + 1.0) - xx;
  const double hi = xx - fl;
  const double gp = fma(tf[ix], lo, tf[ix + 1] * hi);
  return xx < (double)(TABLE_N - 1) ? gp : 0.0;
}

// Exact kernel var_s exp(-arg) with the per-element cutoff arg >= exact_cut -> 0.
__device__ __forceinline__ double s_exact_f64(double dx, double dy, double dz,
                                              const KernelConsts& k) {
  const double arg = k.c_perp * (dx * dx + dy * dy) + k.c_para * (dz * dz);
  return arg < k.exact_cut ? k.var_s * exp(-arg) : 0.0;
}

template <int EVAL>
__device__ __forceinline__ double s_eval_f64(double dx, double dy, double dz,
                                             const KernelConsts& k, const double* tf) {
  if (EVAL == DS_EVAL_TABLE) return s_table_f64(dx, dy, dz, k, tf);
  return s_exact_f64(dx, dy, dz, k);
}

// exp(-a) for 0 <= a <= 700, written from the mathematics for the FP64 pair
// kernels (about 11 FP64 instructions against ~44 for the general exp):
//   k = round(32 a / ln 2),  r = a - k ln2/32  (|r| <= ln2/64, Cody-Waite with
//   a 32-bit high part so k * C_HI is exact for k < 2^21),
//   exp(-a) = 2^-(k >> 5) * 2^-((k & 31)/32) * exp(-r),
// exp(-r) by its Taylor series through degree 6 (truncation < 4e-18 for
// |r| <= ln2/64), 2^-(j/32) from a 32-entry table ``tab`` (tab[j] =
// exp2(-j/32.0)), the power of two applied to the exponent field.  Measured
// error below 4e-16 relative on [0, 45].
__device__ __forceinline__ double exp_neg_f64(double a, const double* tab) {
  const double M = 6755399441055744.0;         // 1.5 * 2^52
  const double K32_LN2 = 46.16624130844683;    // 32 / ln 2
  const double C_HI = 0.02166084938653512;     // ln2/32, 32 significant bits
  const double C_LO = 5.9631716539705866e-12;  // ln2/32 - C_HI
  const double t = fma(a, K32_LN2, M);
  const int k = __double2loint(t);
  const double kd = t - M;
  double r = fma(-kd, C_HI, a);
  r = fma(-kd, C_LO, r);
  const double s = -r;
  double p = fma(s, 1.0 / 720.0, 1.0 / 120.0);
  p = fma(p, s, 1.0 / 24.0);
  p = fma(p, s, 1.0 / 6.0);
  p = fma(p, s, 0.5);
  p = fma(p, s, 1.0);
  p = fma(p, s, 1.0);
  const double v = p * tab[k & 31];
  return __longlong_as_double(__double_as_longlong(v) - ((long long)(k >> 5) << 52));
}

// Sub-tile / tile box test: true when the nearest corners of two boxes
// (lo x, y, z, hi x, y, z in raw coordinates) are inside the cutoff.
__device__ __forceinline__ bool boxes_interact(const double* __restrict__ bi,
                                               const double* __restrict__ bj, double c_perp,
                                               double c_para, double cut) {
  const double dx = fmax(0.0, fmax(bi[0] - bj[3], bj[0] - bi[3]));
  const double dy = fmax(0.0, fmax(bi[1] - bj[4], bj[1] - bi[4]));
  const double dz = fmax(0.0, fmax(bi[2] - bj[5], bj[2] - bi[5]));
  return c_perp * (dx * dx + dy * dy) + c_para * dz * dz < cut;
}

}  // namespace ds
