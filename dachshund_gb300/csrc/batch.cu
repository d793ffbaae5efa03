// Batched solves: many independent sub-volume chunks of uneven size, each
// with n_rhs right-hand sides (noise realisations of the data), solved
// together by the reliable-update mixed-precision PCG of mixed.cu with
// per-(chunk, RHS) scalars and convergence flags.  The chunks share nothing
// but the launches: every reduction is segmented by chunk, and a chunk whose
// right-hand sides have all converged is skipped by every kernel.
//
// One iteration (captured once as a CUDA graph and replayed):
//   MV   q = A32 p for every RHS; persistent launch pulling (row tile, RHS
//        block) items heaviest-first from a work queue; the S value of a pair
//        is generated once per item and applied to RB right-hand sides
//   S1   alpha = r.z / p.q per (chunk, RHS)
//   U2   x_c += alpha p; r -= alpha q; z = r / pd; partial r.z, r.r per tile
//   S2   new r.z, |r|, beta; hold the RHS that want a reliable update; the
//        chunk updates once all its active RHS are held
//   U3   p = z + beta p (RHS still iterating)
//   U4   x += x_c in FP64; x_c = 0 (update pending)
//   R5   r64 = b - A x in FP64 for chunks with an update pending
//   U6   r = float(r64); z = r / pd; partial r.z, |r64|^2
//   S6   FP64 stopping test, restart of the recurrence, beta
//   U7   p = z + beta p after an update;  S7 clears the update flags
// The host replays the graph and reads the number of active chunks every
// 8 iterations.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <tuple>
#include <vector>

#include "ds_batch.h"
#include "ds_tc.cuh"
#include "ds_device.cuh"
#include "ds_ff.cuh"

namespace ds {
namespace {

constexpr int STALL_ITERS = 30;  // iterations without halving the recurrence residual

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// ---- set-up ------------------------------------------------------------------

__global__ void k_offset_perm(int n, const int* __restrict__ in, int offset,
                              int* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = in[i] >= 0 ? in[i] + offset : -1;
}

__global__ void k_offset_int(long long n, const int* __restrict__ in, int offset,
                             int* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = in[i] + offset;
}

// Operator coefficients of every pixel (the single-operator conventions:
// SN: wl = 1, e = N, Jacobi var_s + N;  W: wl = w, e = 1, Jacobi w^2 var_s + 1)
// and their FP32 counterparts (row factor with var_s and, for the EXPANDED
// formula, 2^-|xi|^2 folded in).
__global__ void k_batch_coeffs(int n_pad, int form, double var_s, int expanded,
                               const int* __restrict__ perm, const double* __restrict__ rec,
                               const float4* __restrict__ xi, double* __restrict__ wl,
                               double* __restrict__ e, double* __restrict__ pdiag,
                               float* __restrict__ rowf, float* __restrict__ colw,
                               float* __restrict__ ediag, float* __restrict__ pd32) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_pad) return;
  const int p = perm[i];
  double w = 0.0, ee = 0.0, pdv = 1.0;
  if (p >= 0) {
    const double f = rec[(size_t)p * 5 + 3];
    if (form == DS_FORM_SN) {
      w = 1.0;
      ee = f;
      pdv = __dadd_rn(var_s, f);
    } else {
      w = f;
      ee = 1.0;
      pdv = __dadd_rn(__dmul_rn(__dmul_rn(f, f), var_s), 1.0);
    }
  }
  wl[i] = w;
  e[i] = ee;
  pdiag[i] = pdv;
  const double scale = expanded ? exp2(-(double)xi[i].w) : 1.0;
  rowf[i] = (float)(w * var_s * scale);
  colw[i] = (float)w;
  ediag[i] = (float)ee;
  pd32[i] = (float)pdv;
}

// ---- FP32 multi-RHS matvec on the CUDA cores ------------------------------------

// Work item k: row tile row_order[k / nblk], right-hand sides
// [(k % nblk) RB, +RB).  One row per thread; the 128 columns of a column
// tile are staged with their RB weighted RHS values; each warp runs only the
// column sub-tiles its row sub-tile interacts with.  q = rowf acc + ediag p,
// and the tile's p.q per RHS goes to part[t][r] (FP64 sum of FP32 products).
template <int FORMULA, int RB>
__global__ void __launch_bounds__(TILE) k_batch_mv_f32(BatchF32Args a) {
  __shared__ float4 sc[TILE];
  __shared__ __align__(16) float su[TILE * RB];
  __shared__ int s_item;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int R = a.n_rhs;
  const int nblk = R / RB;
  const int n_items = a.n_row_tiles * nblk;
  for (;;) {
    __syncthreads();  // previous item's shared data fully consumed
    if (tid == 0) s_item = (int)atomicAdd(a.work, 1u);
    __syncthreads();
    const int item = s_item;
    if (item >= n_items) break;
    const int t = a.row_order[item / nblk];
    const int r0 = (item % nblk) * RB;
    if (a.chunk_done[a.tile_chunk[t]]) continue;
    const int i = t * TILE + tid;
    const float4 me = a.xi[i];
    const float4 ot = a.orig[t];
    float acc[RB];
#pragma unroll
    for (int r = 0; r < RB; ++r) acc[r] = 0.f;
    const int p0 = a.row_ptr[t], p1 = a.row_ptr[t + 1];
    unsigned n_sub = 0;  // column sub-tiles this warp evaluates (profiling)
    for (int p = p0; p < p1; ++p) {
      const int ct = a.cols[p];
      const int j = ct * TILE + tid;
      __syncthreads();
      {
        const float4 oc = a.orig[ct];
        const float4 qj = a.xi[j];
        const float zx = qj.x - (ot.x - oc.x), zy = qj.y - (ot.y - oc.y);
        const float zz = qj.z - (ot.z - oc.z);
        if (FORMULA == F32_EXPANDED)
          sc[tid] = make_float4(2.f * zx, 2.f * zy, 2.f * zz, -fmaf(zx, zx, fmaf(zy, zy, zz * zz)));
        else
          sc[tid] = make_float4(zx, zy, zz, 0.f);
        const float cw = a.colw[j];
        const float* pj = a.p + (size_t)j * R + r0;
        if constexpr (RB % 4 == 0) {
#pragma unroll
          for (int r4 = 0; r4 < RB / 4; ++r4) {
            const float4 u = reinterpret_cast<const float4*>(pj)[r4];
            reinterpret_cast<float4*>(su + tid * RB)[r4] =
                make_float4(cw * u.x, cw * u.y, cw * u.z, cw * u.w);
          }
        } else {
#pragma unroll
          for (int r = 0; r < RB; ++r) su[tid * RB + r] = cw * pj[r];
        }
      }
      const unsigned m = (a.mask[p] >> (4 * warp)) & 0xFu;
      n_sub += __popc(m);
      __syncthreads();
      for (int cs = 0; cs < TILE / SUBTILE; ++cs) {
        if (!((m >> cs) & 1u)) continue;
#pragma unroll 2
        for (int jj = cs * SUBTILE; jj < cs * SUBTILE + SUBTILE; ++jj) {
          const float4 c4 = sc[jj];
          float t2;
          if (FORMULA == F32_EXPANDED) {
            t2 = fmaf(me.x, c4.x, c4.w);
            t2 = fmaf(me.y, c4.y, t2);
            t2 = fmaf(me.z, c4.z, t2);
          } else {
            const float dx = me.x - c4.x, dy = me.y - c4.y, dz = me.z - c4.z;
            t2 = -fmaf(dx, dx, fmaf(dy, dy, dz * dz));
          }
          const float s = ex2_approx(t2);
          if constexpr (RB % 4 == 0) {
            const float4* u4 = reinterpret_cast<const float4*>(su + jj * RB);
#pragma unroll
            for (int r4 = 0; r4 < RB / 4; ++r4) {
              const float4 u = u4[r4];
              acc[4 * r4 + 0] = fmaf(s, u.x, acc[4 * r4 + 0]);
              acc[4 * r4 + 1] = fmaf(s, u.y, acc[4 * r4 + 1]);
              acc[4 * r4 + 2] = fmaf(s, u.z, acc[4 * r4 + 2]);
              acc[4 * r4 + 3] = fmaf(s, u.w, acc[4 * r4 + 3]);
            }
          } else {
#pragma unroll
            for (int r = 0; r < RB; ++r) acc[r] = fmaf(s, su[jj * RB + r], acc[r]);
          }
        }
      }
    }
    if (a.prof_pairs && (tid & 31) == 0)
      atomicAdd(a.prof_pairs, (unsigned long long)n_sub * SUBTILE * SUBTILE * RB);
    const float rf = a.rowf[i], ed = a.ediag[i];
    __syncthreads();  // su is reused for the p.q products
#pragma unroll
    for (int r = 0; r < RB; ++r) {
      const size_t k = (size_t)i * R + r0 + r;
      const float pv = a.p[k];
      const float qv = fmaf(rf, acc[r], ed * pv);
      a.q[k] = qv;
      su[tid * RB + r] = pv * qv;
    }
    __syncthreads();
    if (tid < RB) {
      double s = 0.0;
      for (int k = 0; k < TILE; ++k) s += (double)su[k * RB + tid];
      a.part[(size_t)t * R + r0 + tid] = s;
    }
  }
}

// ---- FP64-accurate multi-RHS residual ---------------------------------------------

// u = var_s wl x of the chunks with an update pending, as an unevaluated
// float pair (hi = float(u), lo = float(u - hi)): about 48 significant bits.
__global__ void k_resid_prep(int R, double var_s, const int* __restrict__ tile_chunk,
                             const int* __restrict__ chunk_done,
                             const int* __restrict__ chunk_update, const double* __restrict__ wl,
                             const double* __restrict__ xv, float2* __restrict__ uu) {
  const int t = blockIdx.x;
  const int c = tile_chunk[t];
  if (chunk_done[c] || !chunk_update[c]) return;
  const size_t base = (size_t)t * TILE * R;
  for (int k = threadIdx.x; k < TILE * R; k += blockDim.x) {
    const double u = var_s * wl[t * TILE + k / R] * xv[base + k];
    const float h = __double2float_rn(u);
    uu[base + k] = make_float2(h, __double2float_rn(u - (double)h));
  }
}

// s (0 or a normal number in [2^-100, 1]) as hi + lo floats: hi keeps the
// top 24 significand bits of s exactly (bit operations, no conversion), lo is
// the rounded remainder; values below 2^-100 count as 0.
__device__ __forceinline__ void split_f64(double s, float& h, float& l) {
  const long long bits = __double_as_longlong(s);
  const long long hb = bits & ~((1ll << 29) - 1);
  const int fexp = (int)((hb >> 52) & 0x7FF) - 1023 + 127;
  const float hf = __int_as_float((int)((hb >> 29) & 0x7FFFFF) | (fexp << 23));
  const float lf = __double2float_rn(s - __longlong_as_double(hb));
  const bool tiny = !(s >= 7.888609052210118e-31);  // 2^-100
  h = tiny ? 0.f : hf;
  l = tiny ? 0.f : lf;
}

// (ah, al) += (sh + sl) (uh + ul): the product's rounding error from an FMA,
// the cross terms in FP32, Knuth's two-sum for the high part.  About 12
// FP32 operations; every operation rounds as written (no contraction).
__device__ __forceinline__ void df_mac(float& ah, float& al, float sh, float sl, float uh,
                                       float ul) {
  const float p = __fmul_rn(sh, uh);
  float e = __fmaf_rn(sh, uh, -p);
  e = __fmaf_rn(sh, ul, e);
  e = __fmaf_rn(sl, uh, e);
  const float t = __fadd_rn(ah, p);
  const float bp = __fsub_rn(t, ah);
  const float err = __fadd_rn(__fsub_rn(ah, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  al = __fadd_rn(al, __fadd_rn(err, e));
  ah = t;
}

constexpr float BR_FAR = 16.f;                   // FP32 evaluation at or beyond this argument
constexpr float BR_LOG2E = 1.4426950408889634f;  // log2(e)

__device__ __forceinline__ float ex2_br(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// r64 = b - A x for the chunks with an update pending; work items as in the
// FP32 matvec.  One row per thread.  The exact kernel value of a pair is
// computed once per item and applied to RB right-hand sides, accumulated as
// float pairs on the FP32 pipe (about 44 significant bits, far below the
// 1e-8 relative residual it certifies).  With FF (the default: exact kernel,
// cutoff <= 60) the kernel value itself is a float-pair evaluation
// (ds_ff.cuh) from float-pair scaled coordinates; otherwise it is FP64 (the
// argument rounded as in the single-operator FP64 kernel, exp_neg_f64) split
// into a float pair.  GB300 runs FP64 at 1/64 of the FP32 rate, which is why
// neither the kernel value nor the accumulation stays in FP64.  Warp-private
// staging of the column sub-tiles the warp's rows interact with; the (hi,
// lo) u values padded so that the staging stores avoid bank conflicts.
// With FF, a column whose 32 rows (the warp) all lie at argument >= 16 is
// evaluated in FP32 (a term is then at most e^-16 = 1.1e-7 of var_s |u|,
// evaluated to ~2e-6 relative, as in k_pair_ff_resid):
// one ex2 and one FMA per right-hand side into separate FP32 accumulators,
// against the float-pair kernel value and float-pair multiply-adds.  (At 32
// right-hand sides per item the extra accumulators spill a few registers at
// 3 CTAs per SM; that still beats 2 CTAs per SM without spills and 16
// right-hand sides per item on the 512-chunk batch.)
template <int RB, bool FF>
__global__ void __launch_bounds__(TILE, 3) k_batch_resid_f64(BatchF64Args a) {
  constexpr int ROWF = 2 * RB + 4;  // floats per staged column
  extern __shared__ float4 resid_dyn[];
  float* ustage = reinterpret_cast<float*>(resid_dyn);  // [TILE / 32][SUBTILE][ROWF]
  __shared__ double sw[FF ? 1 : TILE / 32][3][SUBTILE];
  __shared__ float sf[FF ? TILE / 32 : 1][6][SUBTILE];
  __shared__ double tf[32];
  __shared__ float tab_h[32], tab_l[32];
  __shared__ int s_item;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid < 32) {
    tf[tid] = exp2(-(double)tid / 32.0);
    const ff v = ff_from_double(tf[tid]);
    tab_h[tid] = v.h;
    tab_l[tid] = v.l;
  }
  const KernelConsts kc = a.kc;
  const float cut = (float)kc.exact_cut;
  const int R = a.n_rhs;
  const int nblk = R / RB;
  const int n_items = a.n_row_tiles * nblk;
  float* suw = ustage + warp * SUBTILE * ROWF;
  for (;;) {
    __syncthreads();
    if (tid == 0) s_item = (int)atomicAdd(a.work, 1u);
    __syncthreads();
    const int item = s_item;
    if (item >= n_items) break;
    const int t = a.row_order[item / nblk];
    const int r0 = (item % nblk) * RB;
    const int c = a.tile_chunk[t];
    if (a.chunk_done[c] || !a.chunk_update[c]) continue;
    const int i = t * TILE + tid;
    const double xi = a.x[i], yi = a.y[i], zi = a.z[i];
    float ah[RB], al[RB], af[RB];
#pragma unroll
    for (int r = 0; r < RB; ++r) ah[r] = al[r] = af[r] = 0.f;
    unsigned n_sub = 0;
    for (int p = a.row_ptr[t]; p < a.row_ptr[t + 1]; ++p) {
      const unsigned m = (a.mask[p] >> (4 * warp)) & 0xFu;
      if (!m) continue;
      n_sub += __popc(m);
      const int ct = a.cols[p];
      ff Yx{0.f, 0.f}, Yy{0.f, 0.f}, Yz{0.f, 0.f};
      if constexpr (FF) {
        // this row relative to the column tile's origin, scaled
        Yx = ff_from_double(xi * a.ff.sp - a.ff.orig[3 * ct + 0]);
        Yy = ff_from_double(yi * a.ff.sp - a.ff.orig[3 * ct + 1]);
        Yz = ff_from_double(zi * a.ff.sq - a.ff.orig[3 * ct + 2]);
      }
      for (int cs = 0; cs < TILE / SUBTILE; ++cs) {
        if (!((m >> cs) & 1u)) continue;
        const int j = ct * TILE + cs * SUBTILE + lane;
        __syncwarp();
        if constexpr (FF) {
          const float2 cx = a.ff.fx[j], cy = a.ff.fy[j], cz = a.ff.fz[j];
          sf[warp][0][lane] = cx.x;
          sf[warp][1][lane] = cx.y;
          sf[warp][2][lane] = cy.x;
          sf[warp][3][lane] = cy.y;
          sf[warp][4][lane] = cz.x;
          sf[warp][5][lane] = cz.y;
        } else {
          sw[warp][0][lane] = a.x[j];
          sw[warp][1][lane] = a.y[j];
          sw[warp][2][lane] = a.z[j];
        }
        const float2* src = a.uu + (size_t)j * R + r0;
        float2* dst = reinterpret_cast<float2*>(suw + lane * ROWF);
#pragma unroll
        for (int r = 0; r < RB; ++r) dst[r] = src[r];
        __syncwarp();
#pragma unroll 1
        for (int jj = 0; jj < SUBTILE; ++jj) {
          float sh, sl;
          if constexpr (FF) {
            const float dx = (Yx.h - sf[warp][0][jj]) + (Yx.l - sf[warp][1][jj]);
            const float dy = (Yy.h - sf[warp][2][jj]) + (Yy.l - sf[warp][3][jj]);
            const float dz = (Yz.h - sf[warp][4][jj]) + (Yz.l - sf[warp][5][jj]);
            const float d2f = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            if (__all_sync(0xffffffffu, d2f >= BR_FAR)) {
              if (d2f < cut) {
                const float g = ex2_br(-d2f * BR_LOG2E);
                const float2* u2 = reinterpret_cast<const float2*>(suw + jj * ROWF);
#pragma unroll
                for (int r = 0; r < RB; ++r) af[r] = fmaf(g, u2[r].x, af[r]);
              }
              continue;
            }
            const ff d2 = ff_dist2(Yx, Yy, Yz, ff{sf[warp][0][jj], sf[warp][1][jj]},
                                   ff{sf[warp][2][jj], sf[warp][3][jj]},
                                   ff{sf[warp][4][jj], sf[warp][5][jj]});
            if (!(d2.h < cut)) continue;  // warp-divergent skip of a zero term
            const ff g = ff_exp_neg(d2, tab_h, tab_l);
            sh = g.h;
            sl = g.l;
          } else {
            const double dx = xi - sw[warp][0][jj], dy = yi - sw[warp][1][jj];
            const double dz = zi - sw[warp][2][jj];
            const double arg = fma(kc.c_perp, fma(dx, dx, dy * dy), kc.c_para * (dz * dz));
            const double g = arg < kc.exact_cut ? exp_neg_f64(arg, tf) : 0.0;
            split_f64(g, sh, sl);
          }
          const float2* u2 = reinterpret_cast<const float2*>(suw + jj * ROWF);
#pragma unroll
          for (int r = 0; r < RB; ++r) {
            const float2 u = u2[r];
            df_mac(ah[r], al[r], sh, sl, u.x, u.y);
          }
        }
      }
    }
    if (a.prof_pairs && lane == 0)
      atomicAdd(a.prof_pairs, (unsigned long long)n_sub * SUBTILE * SUBTILE * RB);
    const double wli = a.wl[i], ei = a.e[i];
#pragma unroll
    for (int r = 0; r < RB; ++r) {
      const size_t k = (size_t)i * R + r0 + r;
      const double acc = ((double)ah[r] + (double)al[r]) + (double)af[r];
      a.r64[k] = a.b[k] - (wli * acc + ei * a.xv[k]);
    }
  }
}

// Float-pair scaled coordinates of the batch's pixels, relative to the first
// pixel of their tile (the tile origin), and the scaled origins.
__global__ void k_ff_points_batch(int n_pad, const double* __restrict__ x,
                                  const double* __restrict__ y, const double* __restrict__ z,
                                  double sp, double sq, float2* __restrict__ fx,
                                  float2* __restrict__ fy, float2* __restrict__ fz,
                                  double* __restrict__ orig) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_pad) return;
  const int t0 = (i / TILE) * TILE;
  const double ox = x[t0] * sp, oy = y[t0] * sp, oz = z[t0] * sq;
  const ff X = ff_from_double(x[i] * sp - ox), Y = ff_from_double(y[i] * sp - oy);
  const ff Z = ff_from_double(z[i] * sq - oz);
  fx[i] = make_float2(X.h, X.l);
  fy[i] = make_float2(Y.h, Y.l);
  fz[i] = make_float2(Z.h, Z.l);
  if (i == t0) {
    orig[3 * (i / TILE) + 0] = ox;
    orig[3 * (i / TILE) + 1] = oy;
    orig[3 * (i / TILE) + 2] = oz;
  }
}

// ---- per-(pixel, RHS) vector kernels: one CTA per tile, thread = RHS ------------

struct BV {
  int R;
  const int* tile_chunk;
  const int* chunk_done;
  const int* need;      // per (chunk, RHS): update pending
  const int* hold;      // per (chunk, RHS): waiting for the chunk's update
  const int* done;      // per (chunk, RHS)
  const double* alpha;  // per (chunk, RHS)
  const double* beta;
};

// MODE 0 (U2): x_c += alpha p; r -= alpha q; z = r / pd.
// MODE 1 (U6): r = float(r64); z = r / pd (update pending).
// MODE 2 (init): r = float(b); z = r / pd; p = z; x_c = 0.
// Partials per (tile, RHS): r.z at [t][r], |r|^2 at [t][R + r] (FP64 r64 in
// modes 1 and 2).
template <int MODE>
__global__ void k_bu_update(BV v, float* __restrict__ xc, float* __restrict__ rr,
                            float* __restrict__ z, float* __restrict__ p,
                            const float* __restrict__ q, const float* __restrict__ pd,
                            const double* __restrict__ r64, double* __restrict__ part) {
  const int t = blockIdx.x;
  const int c = v.tile_chunk[t];
  const int r = threadIdx.x;
  if (r >= v.R) return;
  const int cr = c * v.R + r;
  if (MODE != 2 && (v.chunk_done[c] || v.done[cr])) return;
  if (MODE == 0 && v.hold[cr]) return;
  if (MODE == 1 && !v.need[cr]) return;
  const float alpha = MODE == 0 ? (float)v.alpha[cr] : 0.f;
  double srz = 0.0, srr = 0.0;
  for (int k = 0; k < TILE; ++k) {
    const int i = t * TILE + k;
    const size_t ir = (size_t)i * v.R + r;
    float ri;
    double rd;
    if (MODE == 0) {
      xc[ir] = fmaf(alpha, p[ir], xc[ir]);
      ri = fmaf(-alpha, q[ir], rr[ir]);
      rd = (double)ri;
    } else {
      rd = r64[ir];
      ri = (float)rd;
      if (MODE == 2) xc[ir] = 0.f;
    }
    rr[ir] = ri;
    const float zi = ri / pd[i];
    z[ir] = zi;
    if (MODE == 2) p[ir] = zi;
    srz = fma((double)ri, (double)zi, srz);
    srr = fma(rd, rd, srr);
  }
  part[(size_t)t * 2 * v.R + r] = srz;
  part[(size_t)t * 2 * v.R + v.R + r] = srr;
}

// MODE 0 (U3): p = z + beta p where the RHS iterates on (not held).
// MODE 1 (U7): the same where an update was made.
template <int MODE>
__global__ void k_bu_dir(BV v, const float* __restrict__ z, float* __restrict__ p) {
  const int t = blockIdx.x;
  const int c = v.tile_chunk[t];
  const int r = threadIdx.x;
  if (r >= v.R || v.chunk_done[c]) return;
  const int cr = c * v.R + r;
  if (v.done[cr]) return;
  if (MODE == 0 && (v.need[cr] || v.hold[cr])) return;
  if (MODE == 1 && !v.need[cr]) return;
  const float beta = (float)v.beta[cr];
  for (int k = 0; k < TILE; ++k) {
    const size_t ir = (size_t)(t * TILE + k) * v.R + r;
    p[ir] = fmaf(beta, p[ir], z[ir]);
  }
}

// U4: x += x_c (FP64); x_c = 0 where an update is pending.
__global__ void k_bu_fold(BV v, double* __restrict__ x, float* __restrict__ xc) {
  const int t = blockIdx.x;
  const int c = v.tile_chunk[t];
  const int r = threadIdx.x;
  if (r >= v.R || v.chunk_done[c]) return;
  const int cr = c * v.R + r;
  if (!v.need[cr] || v.done[cr]) return;
  for (int k = 0; k < TILE; ++k) {
    const size_t ir = (size_t)(t * TILE + k) * v.R + r;
    x[ir] += (double)xc[ir];
    xc[ir] = 0.f;
  }
}

// ---- per-(chunk, RHS) scalar kernels: one CTA per chunk, thread = RHS ------------

// Sum over the chunk's tiles in tile order (deterministic).
__device__ __forceinline__ double chunk_sum(const double* part, int t0, int t1, int stride,
                                            int off) {
  double s = 0.0;
  for (int t = t0; t < t1; ++t) s += part[(size_t)t * stride + off];
  return s;
}

// MODE 0 (S1): alpha = r.z / p.q.
// MODE 1 (S2): new r.z and |r|, beta.  A right-hand side whose recurrence
//              residual fell by delta since its last update, reached tol |b|,
//              stagnated (did not halve in STALL_ITERS iterations; the update
//              then restarts with beta = 0) or hit the iteration cap is held
//              (it stops iterating); once
//              every active RHS of the chunk is held the chunk takes an
//              update.  The FP64 residual of a chunk costs about the same for
//              one RHS as for all, so the chunk's updates stay in step and
//              their number stays that of one solve.
// MODE 2 (S6): FP64 residual: stop (converged / cap) or restart.
// MODE 3 (init): |b|, tol |b|, flags.
// MODE 4 (S7): clear the update flags.
// A chunk with no active RHS left is marked done and leaves the active count.
template <int MODE>
__global__ void k_bs(BatchState s, const double* __restrict__ part) {
  const int c = blockIdx.x, r = threadIdx.x;
  const int R = s.R;
  __shared__ int any_active, any_iterating;
  if (threadIdx.x == 0) {
    any_active = 0;
    any_iterating = 0;
  }
  __syncthreads();
  if (MODE != 3 && s.chunk_done[c]) return;  // uniform over the block
  const int cr = c * R + r;
  if (r < R) {
    const int t0 = s.chunk_tile0[c], t1 = s.chunk_tile0[c + 1];
    if (MODE == 0) {
      if (!s.done[cr] && !s.hold[cr]) s.alpha[cr] = s.rz[cr] / chunk_sum(part, t0, t1, R, r);
    } else if (MODE == 1) {
      if (!s.done[cr] && !s.hold[cr]) {
        const double rz = chunk_sum(part, t0, t1, 2 * R, r);
        const double rn = sqrt(chunk_sum(part, t0, t1, 2 * R, R + r));
        s.rz_old[cr] = s.rz[cr];
        s.rz[cr] = rz;
        const int it = ++s.iter[cr];
        s.rmax[cr] = fmax(s.rmax[cr], rn);
        s.beta[cr] = rz / s.rz_old[cr];
        if (rn < 0.5 * s.rbest[cr]) {
          s.rbest[cr] = rn;
          s.it_best[cr] = it;
        }
        // stagnation: the recurrence residual has not halved for STALL_ITERS
        // iterations (the FP32 / BF16 operator's rounding can stall CG near
        // the tolerance); the update restarts the recurrence from scratch
        const int stall = it - s.it_best[cr] >= STALL_ITERS;
        if (stall) s.stalled[cr] = 1;
        if (rn < s.delta * s.rmax[cr] || rn <= s.tol_norm_b[cr] || it >= s.max_iter || stall)
          s.hold[cr] = 1;
        else
          any_iterating = 1;
      }
    } else if (MODE == 2) {
      if (!s.done[cr] && s.need[cr]) {
        const double rz = chunk_sum(part, t0, t1, 2 * R, r);
        const double rt = sqrt(chunk_sum(part, t0, t1, 2 * R, R + r));
        s.rtrue[cr] = rt;
        ++s.n_updates[cr];
        s.hold[cr] = 0;
        if (rt <= s.tol_norm_b[cr]) {
          s.done[cr] = 1;
          s.converged[cr] = 1;
        } else if (s.iter[cr] >= s.max_iter) {
          s.done[cr] = 1;
        } else {
          s.rz[cr] = rz;  // rz_old keeps the r.z before the held iteration
          s.beta[cr] = s.stalled[cr] ? 0.0 : rz / s.rz_old[cr];
          s.rmax[cr] = rt;
          s.rbest[cr] = rt;
          s.it_best[cr] = s.iter[cr];
          s.stalled[cr] = 0;
        }
      }
    } else if (MODE == 3) {
      const double rz = chunk_sum(part, t0, t1, 2 * R, r);
      const double rt = sqrt(chunk_sum(part, t0, t1, 2 * R, R + r));
      s.rz[cr] = rz;
      s.rtrue[cr] = s.rmax[cr] = s.rbest[cr] = rt;
      s.it_best[cr] = 0;
      s.stalled[cr] = 0;
      s.norm_b[cr] = rt;
      s.tol_norm_b[cr] = s.tol * rt;
      s.iter[cr] = 0;
      s.n_updates[cr] = 0;
      s.need[cr] = 0;
      s.hold[cr] = 0;
      // b = 0: x = 0 is exact (counted as converged with 0 iterations)
      const int zero = !(rt > 0.0);
      s.converged[cr] = zero;
      s.done[cr] = (zero || s.max_iter <= 0) ? 1 : 0;
    } else {
      s.need[cr] = 0;
    }
    if (!s.done[cr]) {
      any_active = 1;
      if (MODE == 1 && !s.hold[cr]) any_iterating = 1;
    }
  }
  __syncthreads();
  const int update = MODE == 1 && any_active && !any_iterating;
  if (update && r < R && !s.done[cr]) s.need[cr] = 1;
  if (threadIdx.x == 0) {
    if (MODE == 1) s.chunk_update[c] = update;
    if (MODE == 4) s.chunk_update[c] = 0;
    if ((MODE == 2 || MODE == 3) && !any_active) {
      s.chunk_done[c] = 1;
      atomicSub(s.active_chunks, 1);
    }
  }
}

// Caller layout [record][R] -> sorted [i][R]; padding rows get 0.
__global__ void k_scatter_rhs(int n_pad, int R, const int* __restrict__ perm,
                              const double* __restrict__ src, double* __restrict__ dst) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (size_t)n_pad * R) return;
  const int i = (int)(k / R), r = (int)(k % R);
  const int p = perm[i];
  dst[k] = p >= 0 ? src[(size_t)p * R + r] : 0.0;
}

// Sorted [i][R] -> caller [record][R], times w in the W form.
__global__ void k_gather_x(int n_pad, int R, const int* __restrict__ perm,
                           const double* __restrict__ wl, int scale_w,
                           const double* __restrict__ src, double* __restrict__ dst) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (size_t)n_pad * R) return;
  const int i = (int)(k / R), r = (int)(k % R);
  const int p = perm[i];
  if (p >= 0) dst[(size_t)p * R + r] = scale_w ? src[k] * wl[i] : src[k];
}

__global__ void k_fill_f32v(size_t n, float v, float* __restrict__ out) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = v;
}

// Caller [record][R] doubles -> sorted [i][R] floats (0 on padding).
__global__ void k_scatter_f32(int n_pad, int R, const int* __restrict__ perm,
                              const double* __restrict__ src, float* __restrict__ dst) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (size_t)n_pad * R) return;
  const int i = (int)(k / R), r = (int)(k % R);
  const int p = perm[i];
  dst[k] = p >= 0 ? (float)src[(size_t)p * R + r] : 0.f;
}

__global__ void k_gather_f32(int n_pad, int R, const int* __restrict__ perm,
                             const float* __restrict__ src, double* __restrict__ dst) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (size_t)n_pad * R) return;
  const int i = (int)(k / R), r = (int)(k % R);
  const int p = perm[i];
  if (p >= 0) dst[(size_t)p * R + r] = (double)src[k];
}

__global__ void k_rel_resid(int n, const double* __restrict__ rt, const double* __restrict__ nb,
                            double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = nb[i] > 0.0 ? rt[i] / nb[i] : 0.0;
}

inline unsigned blocks_for(size_t n, int nt = 256) { return (unsigned)((n + nt - 1) / nt); }

int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    DS_CUDA(cudaGetDevice(&dev));
    DS_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
  }
  return n;
}

// CTAs of a persistent launch: resident CTAs per SM x SMs (queried once per
// kernel, outside any stream capture), at most one per work item.
template <class K>
int persistent_grid(K kernel, int items) {
  static std::mutex mu;
  static std::map<const void*, int> full;
  std::lock_guard<std::mutex> lk(mu);
  auto it = full.find((const void*)kernel);
  if (it == full.end()) {
    int per_sm = 0;
    DS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, TILE, 0));
    it = full.emplace((const void*)kernel, std::max(per_sm, 1) * sm_count()).first;
  }
  return std::max(1, std::min(items, it->second));
}

template <int F, int RB>
void mv_launch(const BatchF32Args& a, int grid, cudaStream_t st) {
  const int items = a.n_row_tiles * (a.n_rhs / RB);
  if (grid <= 0) grid = persistent_grid(k_batch_mv_f32<F, RB>, items);
  k_batch_mv_f32<F, RB><<<grid, TILE, 0, st>>>(a);
}

template <int RB>
constexpr size_t resid_smem() {
  return (size_t)(TILE / 32) * SUBTILE * (2 * RB + 4) * sizeof(float);
}

template <int RB, bool FF>
void resid_launch_t(const BatchF64Args& a, int grid, cudaStream_t st) {
  static bool attr = false;  // set on the first (uncaptured) launch
  if (!attr) {
    DS_CUDA(cudaFuncSetAttribute(k_batch_resid_f64<RB, FF>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)resid_smem<RB>()));
    attr = true;
  }
  const int items = a.n_row_tiles * (a.n_rhs / RB);
  if (grid <= 0) {
    static int full = 0;
    if (!full) {
      int per_sm = 0;
      DS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &per_sm, k_batch_resid_f64<RB, FF>, TILE, resid_smem<RB>()));
      full = std::max(per_sm, 1) * sm_count();
    }
    grid = std::max(1, std::min(items, full));
  }
  k_batch_resid_f64<RB, FF><<<grid, TILE, resid_smem<RB>(), st>>>(a);
}

template <int RB>
void resid_launch(const BatchF64Args& a, int grid, cudaStream_t st) {
  if (a.ff.fx)
    resid_launch_t<RB, true>(a, grid, st);
  else
    resid_launch_t<RB, false>(a, grid, st);
}

// RHS block of the FP64 residual: the largest of 32, 16, 8, 4, 2, 1 dividing R
// (64 float-pair accumulators per thread would spill).
int resid_block(int R) {
  for (int b : {32, 16, 8, 4, 2})
    if (R % b == 0) return b;
  return 1;
}

}  // namespace

bool batch_rb_supported(int R, int rb) {
  return (rb == 1 || rb == 2 || rb == 4 || rb == 8 || rb == 16 || rb == 32) && R % rb == 0;
}

void launch_batch_mv_f32(const BatchF32Args& a, int formula, int rb, int grid, cudaStream_t st) {
  require(batch_rb_supported(a.n_rhs, rb), "unsupported RHS block");
  DS_CUDA(cudaMemsetAsync(a.work, 0, sizeof(unsigned int), st));
#define DS_MV_CASES(F)                             \
  switch (rb) {                                    \
    case 1: mv_launch<F, 1>(a, grid, st); break;   \
    case 2: mv_launch<F, 2>(a, grid, st); break;   \
    case 4: mv_launch<F, 4>(a, grid, st); break;   \
    case 8: mv_launch<F, 8>(a, grid, st); break;   \
    case 16: mv_launch<F, 16>(a, grid, st); break; \
    default: mv_launch<F, 32>(a, grid, st); break; \
  }
  if (formula == F32_EXPANDED) {
    DS_MV_CASES(F32_EXPANDED)
  } else {
    DS_MV_CASES(F32_DIRECT)
  }
#undef DS_MV_CASES
  DS_CHECK_LAUNCH();
}

void launch_batch_resid_f64(const BatchF64Args& a, int grid, cudaStream_t st) {
  k_resid_prep<<<a.n_row_tiles, 256, 0, st>>>(a.n_rhs, a.kc.var_s, a.tile_chunk, a.chunk_done,
                                               a.chunk_update, a.wl, a.xv, a.uu);
  DS_CHECK_LAUNCH();
  DS_CUDA(cudaMemsetAsync(a.work, 0, sizeof(unsigned int), st));
  switch (resid_block(a.n_rhs)) {
    case 32: resid_launch<32>(a, grid, st); break;
    case 16: resid_launch<16>(a, grid, st); break;
    case 8: resid_launch<8>(a, grid, st); break;
    case 4: resid_launch<4>(a, grid, st); break;
    case 2: resid_launch<2>(a, grid, st); break;
    default: resid_launch<1>(a, grid, st); break;
  }
  DS_CHECK_LAUNCH();
}

// ---- building a batch -------------------------------------------------------------

void batch_build(ds_batch* B, const double* d_rec, const int* sizes) {
  cudaStream_t st = B->ctx->stream;
  const int C = B->n_chunks;
  const double LOG2E = 1.4426950408889634;
  const double sp = std::sqrt(B->kc.c_perp), sq = std::sqrt(B->kc.c_para);
  const double fp_ = std::sqrt(B->kc.c_perp * LOG2E), fq = std::sqrt(B->kc.c_para * LOG2E);
  KernelConsts k32 = B->kc;
  k32.cull_arg = B->inner_cut * (1.0 + 1e-9);
  std::vector<PointSet> ps(C);
  std::vector<F32Points> fp(C);
  std::vector<PairList> pl32(C), pl64(C);
  std::vector<int> tile0(C + 1, 0);
  std::vector<long long> rec0(C + 1, 0);
  double max_a = 0.0;
  long long pairs32 = 0, pairs64 = 0;
  for (int c = 0; c < C; ++c) {
    rec0[c + 1] = rec0[c] + sizes[c];
    build_point_set(ps[c], d_rec + rec0[c] * 5, sizes[c], 5, sp, sp, sq, st);
    build_f32_points(fp[c], ps[c], fp_, fp_, fq, st);
    max_a = std::max(max_a, fp[c].max_a);
    build_pair_list(pl32[c], ps[c], ps[c], k32, st);
    build_pair_list(pl64[c], ps[c], ps[c], B->kc, st);
    tile0[c + 1] = tile0[c] + ps[c].n_tiles;
    pairs32 += pl32[c].n_pairs;
    pairs64 += pl64[c].n_pairs;
  }
  const int T = tile0[C];
  require((long long)T * TILE * std::max(1, B->n_rhs) < (1ll << 40), "batch too large");
  const int NP = T * TILE;
  B->n_tiles = T;
  B->n_pad = NP;
  // 2^|xi|^2 must stay well inside FP32 range for the EXPANDED formula.
  B->formula = max_a <= 60.0 ? F32_EXPANDED : F32_DIRECT;

  auto cat_d = [&](DevBuf<double>& dst, DevBuf<double> PointSet::*m) {
    dst.alloc(NP);
    for (int c = 0; c < C; ++c)
      DS_CUDA(cudaMemcpyAsync(dst.p + (size_t)tile0[c] * TILE, (ps[c].*m).p,
                              (size_t)ps[c].n_pad * sizeof(double), cudaMemcpyDeviceToDevice, st));
  };
  cat_d(B->x, &PointSet::x);
  cat_d(B->y, &PointSet::y);
  cat_d(B->z, &PointSet::z);
  B->xi.alloc(NP);
  B->orig.alloc(T);
  B->perm.alloc(NP);
  for (int c = 0; c < C; ++c) {
    DS_CUDA(cudaMemcpyAsync(B->xi.p + (size_t)tile0[c] * TILE, fp[c].xi.p,
                            (size_t)ps[c].n_pad * sizeof(float4), cudaMemcpyDeviceToDevice, st));
    DS_CUDA(cudaMemcpyAsync(B->orig.p + tile0[c], fp[c].orig.p,
                            (size_t)ps[c].n_tiles * sizeof(float4), cudaMemcpyDeviceToDevice,
                            st));
    k_offset_perm<<<blocks_for(ps[c].n_pad), 256, 0, st>>>(
        ps[c].n_pad, ps[c].perm.p, (int)rec0[c], B->perm.p + (size_t)tile0[c] * TILE);
    DS_CHECK_LAUNCH();
  }

  // Concatenated pair lists: column tiles shifted by the chunk's first tile,
  // row pointers by the pairs before the chunk; launch order heaviest row
  // tile first over the whole batch.
  auto cat_pairs = [&](PairList& dst, std::vector<PairList>& src, long long total,
                       long long& evaluated) {
    evaluated = 0;
    dst.n_rows = T;
    dst.n_pairs = total;
    dst.row_ptr.alloc(T + 1);
    dst.cols.alloc(std::max<long long>(total, 1));
    dst.mask.alloc(std::max<long long>(total, 1));
    std::vector<int> counts(T);
    long long off = 0;
    for (int c = 0; c < C; ++c) {
      const int nt = ps[c].n_tiles;
      require(off + src[c].n_pairs < (1ll << 31), "too many tile pairs");
      k_offset_int<<<blocks_for(nt + 1), 256, 0, st>>>(nt + 1, src[c].row_ptr.p, (int)off,
                                                       dst.row_ptr.p + tile0[c]);
      DS_CHECK_LAUNCH();
      if (src[c].n_pairs > 0) {
        k_offset_int<<<blocks_for(src[c].n_pairs), 256, 0, st>>>(src[c].n_pairs, src[c].cols.p,
                                                                 tile0[c], dst.cols.p + off);
        DS_CHECK_LAUNCH();
        DS_CUDA(cudaMemcpyAsync(dst.mask.p + off, src[c].mask.p,
                                src[c].n_pairs * sizeof(unsigned short),
                                cudaMemcpyDeviceToDevice, st));
      }
      std::vector<int> rp(nt + 1);
      std::vector<unsigned short> mk(src[c].n_pairs);
      DS_CUDA(cudaMemcpyAsync(rp.data(), src[c].row_ptr.p, rp.size() * sizeof(int),
                              cudaMemcpyDeviceToHost, st));
      if (!mk.empty())
        DS_CUDA(cudaMemcpyAsync(mk.data(), src[c].mask.p, mk.size() * sizeof(unsigned short),
                                cudaMemcpyDeviceToHost, st));
      DS_CUDA(cudaStreamSynchronize(st));
      for (int k = 0; k < nt; ++k) counts[tile0[c] + k] = rp[k + 1] - rp[k];
      for (unsigned short m : mk) evaluated += (long long)__builtin_popcount(m) * SUBTILE * SUBTILE;
      off += src[c].n_pairs;
    }
    // Launch order: chunks by decreasing work (the tail of the persistent
    // launch is short), and within a chunk its tiles in order, so that the
    // CTAs running at one time share the chunk's column tiles in L2 (every
    // column tile of a chunk is read by most of its row tiles).
    std::vector<long long> work(C, 0);
    for (int c = 0; c < C; ++c)
      for (int t = tile0[c]; t < tile0[c + 1]; ++t) work[c] += counts[t];
    std::vector<int> corder(C);
    std::iota(corder.begin(), corder.end(), 0);
    std::stable_sort(corder.begin(), corder.end(),
                     [&](int a, int b) { return work[a] > work[b]; });
    std::vector<int> order;
    order.reserve(T);
    for (int c : corder)
      for (int t = tile0[c]; t < tile0[c + 1]; ++t) order.push_back(t);
    dst.row_order.alloc(T);
    DS_CUDA(cudaMemcpyAsync(dst.row_order.p, order.data(), T * sizeof(int),
                            cudaMemcpyHostToDevice, st));
    DS_CUDA(cudaStreamSynchronize(st));
  };
  cat_pairs(B->pairs32, pl32, pairs32, B->eval32);
  cat_pairs(B->pairs64, pl64, pairs64, B->eval64);

  std::vector<int> tc(T);
  for (int c = 0; c < C; ++c)
    for (int t = tile0[c]; t < tile0[c + 1]; ++t) tc[t] = c;
  B->tile_chunk.alloc(T);
  B->chunk_tile0.alloc(C + 1);
  DS_CUDA(cudaMemcpyAsync(B->tile_chunk.p, tc.data(), T * sizeof(int), cudaMemcpyHostToDevice,
                          st));
  DS_CUDA(cudaMemcpyAsync(B->chunk_tile0.p, tile0.data(), (C + 1) * sizeof(int),
                          cudaMemcpyHostToDevice, st));

  B->wl.alloc(NP);
  B->e.alloc(NP);
  B->pdiag.alloc(NP);
  B->rowf.alloc(NP);
  B->colw.alloc(NP);
  B->ediag.alloc(NP);
  B->pd32.alloc(NP);
  k_batch_coeffs<<<blocks_for(NP), 256, 0, st>>>(
      NP, B->form, B->kc.var_s, B->formula == F32_EXPANDED, B->perm.p, d_rec, B->xi.p, B->wl.p,
      B->e.p, B->pdiag.p, B->rowf.p, B->colw.p, B->ediag.p, B->pd32.p);
  DS_CHECK_LAUNCH();

  const size_t NR = (size_t)NP * B->n_rhs;
  for (auto* v : {&B->bv, &B->xv, &B->r64}) v->alloc(NR);
  B->uu.alloc(NR);
  for (auto* v : {&B->p, &B->q, &B->rr, &B->zz, &B->xc}) v->alloc(NR);
  k_fill_f32v<<<blocks_for(NR), 256, 0, st>>>(NR, 0.f, B->p.p);  // defined p for tuning
  DS_CHECK_LAUNCH();
  B->part.alloc((size_t)T * 2 * B->n_rhs);
  const size_t CR = (size_t)C * B->n_rhs;
  for (auto* v : {&B->s_rz, &B->s_rz_old, &B->s_alpha, &B->s_beta, &B->s_rmax, &B->s_rbest,
                  &B->s_rtrue,
                  &B->s_norm_b, &B->s_tol_norm_b})
    v->alloc(CR);
  for (auto* v : {&B->s_iter, &B->s_n_updates, &B->s_need, &B->s_hold, &B->s_done,
                  &B->s_converged, &B->s_it_best, &B->s_stalled})
    v->alloc(CR);
  B->chunk_done.alloc(C);
  B->chunk_update.alloc(C);
  B->active.alloc(1);
  B->work.alloc(2);
  B->err.alloc(1);
  DS_CUDA(cudaMemsetAsync(B->err.p, 0, sizeof(int), st));
  if (ff_usable(B->kc)) {
    FFData& f = B->ffd;
    f.fx.alloc(NP);
    f.fy.alloc(NP);
    f.fz.alloc(NP);
    f.orig.alloc((size_t)3 * T);
    k_ff_points_batch<<<blocks_for(NP), 256, 0, st>>>(NP, B->x.p, B->y.p, B->z.p, sp, sq, f.fx.p,
                                                      f.fy.p, f.fz.p, f.orig.p);
    DS_CHECK_LAUNCH();
    f.view = FFPoints{f.fx.p, f.fy.p, f.fz.p, f.orig.p, sp, sq};
  }
  DS_CUDA(cudaMemsetAsync(B->chunk_done.p, 0, C * sizeof(int), st));
  DS_CUDA(cudaStreamSynchronize(st));
  B->pairs32_total = pairs32;
  B->pairs64_total = pairs64;
}

namespace {

BatchF32Args mv_args(ds_batch* B) {
  BatchF32Args a{};
  a.xi = B->xi.p;
  a.orig = B->orig.p;
  a.row_ptr = B->pairs32.row_ptr.p;
  a.cols = B->pairs32.cols.p;
  a.mask = B->pairs32.mask.p;
  a.row_order = B->pairs32.row_order.p;
  a.n_row_tiles = B->n_tiles;
  a.tile_chunk = B->tile_chunk.p;
  a.chunk_done = B->chunk_done.p;
  a.colw = B->colw.p;
  a.rowf = B->rowf.p;
  a.ediag = B->ediag.p;
  a.n_rhs = B->n_rhs;
  a.p = B->p.p;
  a.q = B->q.p;
  a.part = B->part.p;
  a.work = B->work.p;
  a.formula = B->formula;
  a.panel = B->panel.p;
  a.err = B->err.p;
  a.wait_limit = B->ctx->wait_limit > 0 ? B->ctx->wait_limit : WAIT_CYCLES;
  return a;
}

BatchF64Args resid_args(ds_batch* B) {
  BatchF64Args a{};
  a.kc = B->kc;
  a.x = B->x.p;
  a.y = B->y.p;
  a.z = B->z.p;
  a.wl = B->wl.p;
  a.e = B->e.p;
  a.b = B->bv.p;
  a.xv = B->xv.p;
  a.r64 = B->r64.p;
  a.row_ptr = B->pairs64.row_ptr.p;
  a.cols = B->pairs64.cols.p;
  a.mask = B->pairs64.mask.p;
  a.row_order = B->pairs64.row_order.p;
  a.n_row_tiles = B->n_tiles;
  a.tile_chunk = B->tile_chunk.p;
  a.chunk_done = B->chunk_done.p;
  a.chunk_update = B->chunk_update.p;
  a.n_rhs = B->n_rhs;
  a.work = B->work.p + 1;
  a.uu = B->uu.p;
  a.ff = B->ffd.view;  // fx == nullptr: FP64 kernel value
  return a;
}

BatchState state_args(ds_batch* B, const ds_mixed_params& mp) {
  BatchState s{};
  s.R = B->n_rhs;
  s.tol = mp.tol;
  s.delta = mp.reliable_delta > 0.0 ? mp.reliable_delta : 1e-4;
  s.max_iter = std::max(mp.max_iter, 0);
  s.chunk_tile0 = B->chunk_tile0.p;
  s.rz = B->s_rz.p;
  s.rz_old = B->s_rz_old.p;
  s.alpha = B->s_alpha.p;
  s.beta = B->s_beta.p;
  s.rmax = B->s_rmax.p;
  s.rbest = B->s_rbest.p;
  s.it_best = B->s_it_best.p;
  s.stalled = B->s_stalled.p;
  s.rtrue = B->s_rtrue.p;
  s.norm_b = B->s_norm_b.p;
  s.tol_norm_b = B->s_tol_norm_b.p;
  s.iter = B->s_iter.p;
  s.n_updates = B->s_n_updates.p;
  s.need = B->s_need.p;
  s.hold = B->s_hold.p;
  s.done = B->s_done.p;
  s.converged = B->s_converged.p;
  s.chunk_done = B->chunk_done.p;
  s.chunk_update = B->chunk_update.p;
  s.active_chunks = B->active.p;
  return s;
}

// Autotuner cache: (n_rhs, formula, log2 of the tile count) -> (variant, rb).
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int>, std::pair<int, int>> g_tune;

}  // namespace

// q = A32 p over every chunk not done, with the chosen variant.  With the
// context's profiling on, the launch is timed (kind 1) and its pair x RHS
// products counted.
void batch_mv(ds_batch* B, cudaStream_t st) {
  if (B->variant == BV_TENSOR && !B->panel.p)
    B->panel.alloc(batch_tc_panel_elems(B->n_tiles, B->n_rhs));
  BatchF32Args a = mv_args(B);
  Profiler& pr = B->ctx->prof;
  cudaEvent_t ev = nullptr;
  if (pr.enabled) {
    a.prof_pairs = pr.d_pairs + 1;
    pr.begin(st, &ev);
  }
  if (B->variant == BV_TENSOR)
    launch_batch_mv_tc(a, st);
  else
    launch_batch_mv_f32(a, B->formula, B->rb, B->grid_mv, st);
  if (ev) pr.end(st, ev, 1);
}

bool batch_variant_supported(const ds_batch* B, int variant) {
  if (variant == BV_CUDA_CORE) return true;
  return variant == BV_TENSOR && batch_tc_block(B->n_rhs) != 0;
}

// Raises the code a timed-out wait of the tensor-core kernel left behind.
static void check_tc_error(ds_batch* B) {
  int code = 0;
  DS_CUDA(cudaMemcpyAsync(&code, B->err.p, sizeof(int), cudaMemcpyDeviceToHost, B->ctx->stream));
  DS_CUDA(cudaStreamSynchronize(B->ctx->stream));
  if (code) {
    DS_CUDA(cudaMemsetAsync(B->err.p, 0, sizeof(int), B->ctx->stream));
    throw Error{DS_ERR_TIMEOUT, "tensor-core matvec: an mbarrier wait timed out (code " +
                                 std::to_string(code) + ")"};
  }
}

// r64 = b - A x (FP64) over the chunks flagged in chunk_update (profiled as
// kind 0).
void batch_resid(ds_batch* B, cudaStream_t st) {
  BatchF64Args a = resid_args(B);
  Profiler& pr = B->ctx->prof;
  cudaEvent_t ev = nullptr;
  if (pr.enabled) {
    a.prof_pairs = pr.d_pairs;
    pr.begin(st, &ev);
  }
  launch_batch_resid_f64(a, 0, st);
  if (ev) pr.end(st, ev, 0);
}

void batch_product_f32_dev(ds_batch* B, const double* p_dev, double* q_dev) {
  cudaStream_t st = B->ctx->stream;
  const size_t NR = (size_t)B->n_pad * B->n_rhs;
  if (!B->tuned) batch_autotune(B, false, nullptr);
  k_scatter_f32<<<blocks_for(NR), 256, 0, st>>>(B->n_pad, B->n_rhs, B->perm.p, p_dev, B->p.p);
  DS_CHECK_LAUNCH();
  DS_CUDA(cudaMemsetAsync(B->chunk_done.p, 0, B->n_chunks * sizeof(int), st));
  batch_mv(B, st);
  k_gather_f32<<<blocks_for(NR), 256, 0, st>>>(B->n_pad, B->n_rhs, B->perm.p, B->q.p, q_dev);
  DS_CHECK_LAUNCH();
  if (B->variant == BV_TENSOR) check_tc_error(B);
}

// Times every matvec variant that fits n_rhs on this batch (one warm-up and
// the best of three launches each) and keeps the fastest; the choice is
// cached for batches of the same shape class (n_rhs, formula, log2 tiles).
void batch_autotune(ds_batch* B, bool force, double* best_ms_out) {
  const int R = B->n_rhs;
  int lg = 0;
  while ((1 << (lg + 1)) <= B->n_tiles) ++lg;
  const auto key = std::make_tuple(R, B->formula, lg);
  if (!force) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      B->variant = it->second.first;
      B->rb = it->second.second;
      B->tuned = true;
      return;
    }
  }
  cudaStream_t st = B->ctx->stream;
  DS_CUDA(cudaMemsetAsync(B->chunk_done.p, 0, B->n_chunks * sizeof(int), st));
  cudaEvent_t e0, e1;
  DS_CUDA(cudaEventCreate(&e0));
  DS_CUDA(cudaEventCreate(&e1));
  double best = 1e300;
  int best_rb = 0, best_variant = BV_CUDA_CORE;
  const int rb0 = B->rb;
  auto time_mv = [&]() {
    batch_mv(B, st);
    float t_min = 1e30f;
    for (int k = 0; k < 3; ++k) {
      DS_CUDA(cudaEventRecord(e0, st));
      batch_mv(B, st);
      DS_CUDA(cudaEventRecord(e1, st));
      DS_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      DS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      t_min = std::min(t_min, ms);
    }
    return (double)t_min;
  };
  try {
    B->variant = BV_CUDA_CORE;
    for (int rb : {4, 8, 16, 32}) {
      if (!batch_rb_supported(R, rb)) continue;
      B->rb = rb;
      const double t = time_mv();
      if (t < best) {
        best = t;
        best_rb = rb;
      }
    }
    if (batch_variant_supported(B, BV_TENSOR)) {
      B->variant = BV_TENSOR;
      const double t = time_mv();
      check_tc_error(B);
      if (t < best) {
        best = t;
        best_variant = BV_TENSOR;
      }
    }
  } catch (...) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    B->variant = BV_CUDA_CORE;
    B->rb = rb0;
    throw;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (best_rb == 0) best_rb = batch_rb_supported(R, 2) ? 2 : 1;
  B->variant = best_variant;
  B->rb = best_rb;
  B->tuned = true;
  if (best_ms_out) *best_ms_out = best;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[key] = {B->variant, B->rb};
}

// The device-side loop of the batched solve: counts the iteration just run
// and continues while a chunk is active and fewer than `cap` have run.
__global__ void k_batch_loop(cudaGraphConditionalHandle h, const int* active, int* count,
                             int cap) {
  const int n = ++*count;
  cudaGraphSetConditional(h, (*active > 0 && n < cap) ? 1u : 0u);
}

// The batched solve on device vectors: rhs_dev and x_dev are [record][R] in
// the caller's order (x0 = 0).  Per-(chunk, RHS) results go to the host
// arrays that are given.
void batch_solve_dev(ds_batch* B, const ds_mixed_params& mp, const double* rhs_dev, double* x_dev,
                     int* iters, int* converged, int* n_updates, double* rel_resid,
                     double* seconds) {
  cudaStream_t st = B->ctx->stream;
  const int C = B->n_chunks, R = B->n_rhs, T = B->n_tiles, NP = B->n_pad;
  const size_t NR = (size_t)NP * R;
  if (!B->tuned) batch_autotune(B, false, nullptr);
  k_scatter_rhs<<<blocks_for(NR), 256, 0, st>>>(NP, R, B->perm.p, rhs_dev, B->bv.p);
  DS_CHECK_LAUNCH();
  DS_CUDA(cudaMemsetAsync(B->xv.p, 0, NR * sizeof(double), st));
  DS_CUDA(cudaMemsetAsync(B->chunk_done.p, 0, C * sizeof(int), st));
  DS_CUDA(cudaMemsetAsync(B->chunk_update.p, 0, C * sizeof(int), st));
  const int h_active = C;
  DS_CUDA(cudaMemcpyAsync(B->active.p, &h_active, sizeof(int), cudaMemcpyHostToDevice, st));
  DS_CUDA(cudaStreamSynchronize(st));  // h_active is on this stack frame

  const BatchState S = state_args(B, mp);
  const BV v{R,           B->tile_chunk.p, B->chunk_done.p, B->s_need.p,
             B->s_hold.p, B->s_done.p,     B->s_alpha.p,     B->s_beta.p};
  const int RT = ((R + 31) / 32) * 32;

  cudaEvent_t ev0, ev1;
  DS_CUDA(cudaEventCreate(&ev0));
  DS_CUDA(cudaEventCreate(&ev1));
  DS_CUDA(cudaEventRecord(ev0, st));
  // r = b (x0 = 0), z = M^-1 r, p = z, x_c = 0
  k_bu_update<2><<<T, RT, 0, st>>>(v, B->xc.p, B->rr.p, B->zz.p, B->p.p, nullptr, B->pd32.p,
                                   B->bv.p, B->part.p);
  DS_CHECK_LAUNCH();
  k_bs<3><<<C, RT, 0, st>>>(S, B->part.p);
  DS_CHECK_LAUNCH();

  auto issue_iteration = [&] {
    batch_mv(B, st);                                                                 // MV
    k_bs<0><<<C, RT, 0, st>>>(S, B->part.p);                                         // S1
    DS_CHECK_LAUNCH();
    k_bu_update<0><<<T, RT, 0, st>>>(v, B->xc.p, B->rr.p, B->zz.p, B->p.p, B->q.p,
                                     B->pd32.p, nullptr, B->part.p);                 // U2
    DS_CHECK_LAUNCH();
    k_bs<1><<<C, RT, 0, st>>>(S, B->part.p);                                         // S2
    DS_CHECK_LAUNCH();
    k_bu_dir<0><<<T, RT, 0, st>>>(v, B->zz.p, B->p.p);                               // U3
    DS_CHECK_LAUNCH();
    k_bu_fold<<<T, RT, 0, st>>>(v, B->xv.p, B->xc.p);                                // U4
    DS_CHECK_LAUNCH();
    batch_resid(B, st);                                                              // R5
    k_bu_update<1><<<T, RT, 0, st>>>(v, B->xc.p, B->rr.p, B->zz.p, B->p.p, nullptr,
                                     B->pd32.p, B->r64.p, B->part.p);                // U6
    DS_CHECK_LAUNCH();
    k_bs<2><<<C, RT, 0, st>>>(S, B->part.p);                                         // S6
    DS_CHECK_LAUNCH();
    k_bu_dir<1><<<T, RT, 0, st>>>(v, B->zz.p, B->p.p);                               // U7
    DS_CHECK_LAUNCH();
    k_bs<4><<<C, RT, 0, st>>>(S, B->part.p);                                         // S7
    DS_CHECK_LAUNCH();
  };
  // The first iteration runs eagerly (every kernel and its module loaded
  // outside the capture); the rest replay its graph.  With the context's
  // profiling on, every iteration runs eagerly so that the matvec and the
  // FP64 residual launches can be timed one by one.
  int it = 0;
  if (S.max_iter > 0) {
    issue_iteration();
    it = 1;
  }
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int active = C;
  int replays = 0;
  // A held RHS does not count iterations while the rest of its chunk runs
  // on, so the graph may run more than max_iter times; every active RHS
  // reaches its cap long before this safety bound.
  const long long it_cap = 4ll * S.max_iter + 64;
  if (B->ctx->prof.enabled) {
    for (; it < it_cap && active > 0; ++it) {
      issue_iteration();
      if (it % 8 == 7) {
        DS_CUDA(cudaMemcpyAsync(&active, B->active.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        DS_CUDA(cudaStreamSynchronize(st));
      }
    }
  } else if (it < it_cap) {
    // The rest of the solve is one graph launch: a WHILE conditional node
    // whose body is one iteration followed by k_batch_loop, which counts the
    // iterations on the device and keeps the loop going while a chunk is
    // active and the count is under the cap (so the loop ends by itself).
    const long long launches0 = launch_counter();
    B->loop_it.alloc(1);
    DS_CUDA(cudaMemsetAsync(B->loop_it.p, 0, sizeof(int), st));
    DS_CUDA(cudaGraphCreate(&graph, 0));
    cudaGraphConditionalHandle h;
    cudaGraphNodeParams cp{};
    cudaGraphNode_t node;
    try {
      DS_CUDA(cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault));
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = h;
      cp.conditional.type = cudaGraphCondTypeWhile;
      cp.conditional.size = 1;
      DS_CUDA(cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp));
      cudaGraph_t body = cp.conditional.phGraph_out[0];
      DS_CUDA(cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0,
                                            cudaStreamCaptureModeThreadLocal));
      try {
        issue_iteration();
        k_batch_loop<<<1, 1, 0, st>>>(h, B->active.p, B->loop_it.p, (int)(it_cap - it));
        DS_CHECK_LAUNCH();
      } catch (...) {
        cudaStreamEndCapture(st, &body);
        throw;
      }
      DS_CUDA(cudaStreamEndCapture(st, &body));
    } catch (...) {
      cudaGraphDestroy(graph);
      graph = nullptr;
      cudaEventDestroy(ev0);
      cudaEventDestroy(ev1);
      throw;
    }
    const long long per_iter = launch_counter() - launches0;
    const cudaError_t inst = cudaGraphInstantiate(&exec, graph, 0);
    if (inst != cudaSuccess) {
      cudaGraphDestroy(graph);
      DS_CUDA(inst);
    }
    DS_CUDA(cudaGraphLaunch(exec, st));
    int ran = 0;
    DS_CUDA(cudaMemcpyAsync(&ran, B->loop_it.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    DS_CUDA(cudaStreamSynchronize(st));
    replays = ran;
    // the capture counted one iteration's launches; the loop ran `ran`
    launch_counter() += (long long)(ran - 1) * per_iter;
  }
  DS_CUDA(cudaEventRecord(ev1, st));
  DS_CUDA(cudaStreamSynchronize(st));
  B->graph_replays = replays;
  if (B->variant == BV_TENSOR) check_tc_error(B);
  float ms = 0.f;
  DS_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
  if (seconds) *seconds = ms * 1e-3;
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);

  k_gather_x<<<blocks_for(NR), 256, 0, st>>>(NP, R, B->perm.p, B->wl.p, B->form == DS_FORM_W,
                                             B->xv.p, x_dev);
  DS_CHECK_LAUNCH();
  const size_t CR = (size_t)C * R;
  if (iters)
    DS_CUDA(cudaMemcpyAsync(iters, B->s_iter.p, CR * sizeof(int), cudaMemcpyDeviceToHost, st));
  if (converged)
    DS_CUDA(cudaMemcpyAsync(converged, B->s_converged.p, CR * sizeof(int),
                            cudaMemcpyDeviceToHost, st));
  if (n_updates)
    DS_CUDA(cudaMemcpyAsync(n_updates, B->s_n_updates.p, CR * sizeof(int),
                            cudaMemcpyDeviceToHost, st));
  if (rel_resid) {
    k_rel_resid<<<blocks_for(CR), 256, 0, st>>>((int)CR, B->s_rtrue.p, B->s_norm_b.p,
                                               B->s_rz_old.p);
    DS_CHECK_LAUNCH();
    DS_CUDA(cudaMemcpyAsync(rel_resid, B->s_rz_old.p, CR * sizeof(double),
                            cudaMemcpyDeviceToHost, st));
  }
  DS_CUDA(cudaStreamSynchronize(st));
}

}  // namespace ds
