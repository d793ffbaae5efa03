// Dense paths: the operator A built densely in HBM, the dense FP64 matvec
// used by PCG when the matrix fits, and the closed-form solve (Cholesky) that
// stands in for WFVector{SN,W}::solve_cf (lib/wf_vector.cc:123-155, 276-319).
//
// Dense matvec: A streamed once per product (8 n^2 bytes) by a persistent
// grid over 64 x 2048 blocks, HBM-bound with float-pair arithmetic on the
// FP32 pipe (see the matvec section below).
// Cholesky: right-looking, 32-wide panels: diagonal block in shared memory by
// one CTA, the panel by a triangular solve per row, the trailing lower
// triangle by 64 x 64 tiles (each thread a 4 x 4 block).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "ds_device.cuh"
#include "ds_ops.h"

namespace ds {
namespace {

constexpr int NB = 32;       // Cholesky panel width
constexpr int DTILE = 64;    // trailing-update tile

// A_ij of the operator for every (i, j) < n (row-major, leading dim ld), in
// the order of the given coordinate/coefficient arrays (sorted or caller);
// one row per CTA at a time, coalesced stores.  With ``stats`` it also
// records the entry range that chooses the matvec's arithmetic
// (dense_stats_add, defined with the matvec below).
__device__ __forceinline__ void dense_stats_add(unsigned long long* st, unsigned long long mn,
                                                unsigned long long mx, unsigned neg);

__global__ void k_dense_build(KernelConsts kc, int n, size_t ld, const double* __restrict__ x,
                              const double* __restrict__ y, const double* __restrict__ z,
                              const double* __restrict__ wl, const double* __restrict__ e,
                              const double* __restrict__ table, double* __restrict__ A,
                              unsigned long long* stats) {
  __shared__ double tf[TABLE_N];
  for (int k = threadIdx.x; k < TABLE_N; k += blockDim.x) tf[k] = table[k];
  __syncthreads();
  unsigned long long mn = ~0ull, mx = 0ull;
  unsigned neg = 0;
  for (int i = blockIdx.x; i < n; i += gridDim.x) {
    const double xi = x[i], yi = y[i], zi = z[i], wi = wl[i], ei = e[i];
    double* Ai = A + (size_t)i * ld;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
      const double dx = xi - x[j], dy = yi - y[j], dz = zi - z[j];
      double S;
      if (kc.eval == DS_EVAL_TABLE) {
        S = s_table_f64(dx, dy, dz, kc, tf);
      } else {
        const double arg = kc.c_perp * (dx * dx + dy * dy) + kc.c_para * (dz * dz);
        S = arg < kc.exact_cut ? kc.var_s * exp(-arg) : 0.0;
      }
      const double a = wi * S * wl[j] + (i == j ? ei : 0.0);
      __stcs(Ai + j, a);
      if (stats) {
        const unsigned long long bits = (unsigned long long)__double_as_longlong(a);
        const unsigned long long mag = bits & 0x7fffffffffffffffull;
        if (mag) mn = min(mn, mag);
        mx = max(mx, mag);
        neg |= (unsigned)(bits >> 63) & (mag != 0);
      }
    }
  }
  if (stats) dense_stats_add(stats, mn, mx, neg);
}

// ---- dense matvec ------------------------------------------------------------
//
// q = A v (+ the last CTA's alpha = delta / (dotv . q)) or r = b - A v, A in
// HBM (n x n FP64, row-major, sorted order).  Work items are 64-row x
// 2048-column blocks of A pulled by a persistent grid (CTA count a multiple
// of the SM count); each warp streams 8 rows of its block with 16-byte
// evict-first loads (every byte of A read once per product), and the column
// slice of v is read through L1 (the 8 warps of a CTA share it).  Per-block
// row sums go to a partial buffer; the last block of a row block to finish
// (an atomic count) adds its rows' partials in column-block order, so the
// result does not depend on the finishing order.
//
// Two arithmetics:
//  * FLOAT_PAIR (default): GB300 issues FP64 FMAs at 2 per clock per SM,
//    which caps an FP64 matvec at ~5 TB/s of matrix data, below HBM.  Each
//    FP64 entry is split with integer operations into a head of 24 and a
//    tail of 23 significant bits (exact to 2^-46 relative), multiplied by v
//    as a float pair (v split once per product) with FMA-exact head products,
//    and summed in float-float (Knuth two-sum) on the FP32 pipe; each
//    block's float pair is added in FP64.  About 24 FP32/INT operations per
//    entry against the ~47 the FP32 pipe can issue per HBM entry, so the
//    product runs at the HBM rate.  Valid when every nonzero |A_ij| is in
//    [2^-100, 2^100] (checked when the matrix is built).
//  * FP64: plain FP64 FMAs (the FP64-pipe bound above).

constexpr int DM_WARPS = 8;
constexpr int DM_ROWS = 8;                  // rows per warp
constexpr int DM_RB = DM_WARPS * DM_ROWS;   // rows per work item
constexpr int DM_CW = 2048;                 // columns per work item
constexpr int DM_CTAS_PER_SM = 2;

struct DenseMv {
  int n;     // rows = columns (n_pad, a multiple of 128)
  int nrb;   // row blocks
  int ncb;   // column blocks
  const double* A;
  const double* v;    // FP64 arithmetic
  const float2* vff;  // FLOAT_PAIR arithmetic: v as (head, tail) floats
  const double* b;
  double* out;
  const double* dotv;
  double* part;       // ncb x n row partials
  double* dot_part;   // nrb
  unsigned int* rb_cnt;  // nrb arrival counts (zero between launches)
  unsigned int* cnt;     // row blocks finished (zero between launches)
  PcgState* pcg;
  const int* skip;
  unsigned long long* prof_pairs;
};

// a = h + l to 2^-46 |a| for a = 0 or 2^-100 <= |a| <= 2^100: h holds the
// sign, exponent and top 23 stored mantissa bits; the next 23 bits become a
// float X = 2^(E-23) (1 + q 2^-23) from which the exact power 2^(E-23) is
// subtracted (no int-to-float conversion).  A zero gives h = l = 0.
template <bool SIGNED>
__device__ __forceinline__ void split_f64(unsigned lo, unsigned hi, float& h, float& l) {
  const unsigned body = hi & 0x7fffffffu;
  const int eh = max((int)(body - (896u << 20)), 0);  // float-biased exponent in bits 27..20
  unsigned hb = __funnelshift_l(lo, (unsigned)eh, 3);
  const unsigned yb = (((unsigned)eh << 3) & 0x7f800000u) - (23u << 23);
  const unsigned xb = yb | ((lo >> 6) & 0x7fffffu);
  float lv = __fsub_rn(__uint_as_float(xb), __uint_as_float(yb));
  if (SIGNED) {
    const unsigned sg = hi & 0x80000000u;
    hb |= sg;
    lv = __uint_as_float(__float_as_uint(lv) | sg);
  }
  h = __uint_as_float(hb);
  l = lv;
}

// (sh, sl) += (h + l)(vh + vl), float-float (the l vl term is below 2^-46).
__device__ __forceinline__ void ff_mac(float h, float l, float vh, float vl, float& sh,
                                       float& sl) {
  const float p = __fmul_rn(h, vh);
  float e = __fmaf_rn(h, vh, -p);
  e = __fmaf_rn(h, vl, e);
  e = __fmaf_rn(l, vh, e);
  const float s = __fadd_rn(sh, p);
  const float bb = __fsub_rn(s, sh);
  const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  sl = __fadd_rn(sl, __fadd_rn(err, e));
  sh = s;
}

__device__ __forceinline__ uint4 ld_stream16(const double* p) {
  uint4 r;
  asm volatile("ld.global.nc.L1::no_allocate.L2::256B.v4.u32 {%0, %1, %2, %3}, [%4];"
               : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
               : "l"(p));
  return r;
}

__global__ void k_split_vec(int n, const double* __restrict__ v, float2* __restrict__ vff,
                            const int* skip) {
  if (skip && *skip) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double x = v[i];
    const float h = __double2float_rn(x);
    vff[i] = make_float2(h, __double2float_rn(x - (double)h));
  }
}

template <bool FF, bool SIGNED, bool RESIDUAL, bool DOT>
__global__ void __launch_bounds__(DM_WARPS * 32, DM_CTAS_PER_SM) k_dense_mv(DenseMv a) {
  if (a.skip && *a.skip) return;
  if (a.prof_pairs && blockIdx.x == 0 && threadIdx.x == 0)
    atomicAdd(a.prof_pairs, (unsigned long long)a.n * (unsigned long long)a.n);
  __shared__ double red[DM_WARPS];
  __shared__ int s_last;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n_items = a.nrb * a.ncb;
  for (int item = blockIdx.x; item < n_items; item += gridDim.x) {
    const int rb = item / a.ncb, cb = item - rb * a.ncb;
    const int c0 = cb * DM_CW;
    const int steps = min(DM_CW, a.n - c0) >> 6;  // 64 columns per warp step
    const int r0 = rb * DM_RB + warp * DM_ROWS;
    const double* Ab = a.A + (size_t)r0 * a.n + c0 + 2 * lane;
    float sh[DM_ROWS], sl[DM_ROWS];
    double acc[DM_ROWS];
#pragma unroll
    for (int r = 0; r < DM_ROWS; ++r) {
      sh[r] = sl[r] = 0.f;
      acc[r] = 0.0;
    }
#pragma unroll 2
    for (int s = 0; s < steps; ++s) {
      const int c = c0 + 64 * s + 2 * lane;
      uint4 q[DM_ROWS];
#pragma unroll
      for (int r = 0; r < DM_ROWS; ++r) q[r] = ld_stream16(Ab + (size_t)r * a.n + 64 * s);
      if (FF) {
        const float4 vv = __ldg(reinterpret_cast<const float4*>(a.vff + c));
#pragma unroll
        for (int r = 0; r < DM_ROWS; ++r) {
          float h, l;
          split_f64<SIGNED>(q[r].x, q[r].y, h, l);
          ff_mac(h, l, vv.x, vv.y, sh[r], sl[r]);
          split_f64<SIGNED>(q[r].z, q[r].w, h, l);
          ff_mac(h, l, vv.z, vv.w, sh[r], sl[r]);
        }
      } else {
        const double2 vv = __ldg(reinterpret_cast<const double2*>(a.v + c));
#pragma unroll
        for (int r = 0; r < DM_ROWS; ++r) {
          acc[r] = fma(__hiloint2double((int)q[r].y, (int)q[r].x), vv.x, acc[r]);
          acc[r] = fma(__hiloint2double((int)q[r].w, (int)q[r].z), vv.y, acc[r]);
        }
      }
    }
    // this block's row sums: lane partials in FP64, fixed shuffle tree
#pragma unroll
    for (int r = 0; r < DM_ROWS; ++r) {
      double t = FF ? (double)sh[r] + (double)sl[r] : acc[r];
      for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
      if (lane == 0) a.part[(size_t)cb * a.n + r0 + r] = t;
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(&a.rb_cnt[rb], 1u) == (unsigned)(a.ncb - 1);
    __syncthreads();
    if (s_last) {  // every column block of this row block is in: finish its rows
      __threadfence();
      double dot = 0.0;
      if (tid < DM_RB) {
        const int row = rb * DM_RB + tid;
        double sum = 0.0;
        for (int k = 0; k < a.ncb; ++k) sum += __ldcg(a.part + (size_t)k * a.n + row);
        const double o = RESIDUAL ? a.b[row] - sum : sum;
        a.out[row] = o;
        if (DOT) dot = a.dotv[row] * o;
      }
      if (tid == 0) a.rb_cnt[rb] = 0;
      if (DOT) {
        const double bs = block_sum<DM_WARPS * 32>(dot, red);
        if (tid == 0) a.dot_part[rb] = bs;
        __threadfence();
        __syncthreads();
        if (tid == 0) s_last = atomicAdd(a.cnt, 1u) == (unsigned)(a.nrb - 1);
        __syncthreads();
        if (s_last) {  // the last row block: alpha = delta / (d . q), lib/pcg.h:37
          __threadfence();
          const double dq = reduce_partials<DM_WARPS * 32>(a.dot_part, a.nrb, 1, 0, red);
          if (tid == 0) {
            a.pcg->dq = dq;
            a.pcg->alpha = a.pcg->delta / dq;
            *a.cnt = 0;
          }
        }
      }
    }
    __syncthreads();  // s_last and red are reused by the next item
  }
}

// Folds a thread's entry statistics into stats[0..2]: the smallest nonzero
// and the largest |A_ij| as FP64 bit patterns (which order like the values
// for non-negative numbers) and whether any entry is negative.
__device__ __forceinline__ void dense_stats_add(unsigned long long* st, unsigned long long mn,
                                                unsigned long long mx, unsigned neg) {
  for (int o = 16; o > 0; o >>= 1) {
    mn = min(mn, __shfl_down_sync(0xffffffffu, mn, o));
    mx = max(mx, __shfl_down_sync(0xffffffffu, mx, o));
    neg |= __shfl_down_sync(0xffffffffu, neg, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(st + 0, mn);
    atomicMax(st + 1, mx);
    if (neg) atomicOr(st + 2, 1ull);
  }
}

// ---- Cholesky ------------------------------------------------------------

// Unblocked Cholesky of the b x b diagonal block at (k, k), in shared memory.
__global__ void k_potrf_diag(double* __restrict__ A, size_t ld, int k, int b, int* bad) {
  __shared__ double s[NB][NB + 1];
  const int t = threadIdx.x;  // NB threads, one per row
  for (int c = 0; c < b; ++c) s[t][c] = t < b ? A[(size_t)(k + t) * ld + k + c] : 0.0;
  __syncthreads();
  for (int j = 0; j < b; ++j) {
    if (t == j) {
      const double d = s[j][j];
      if (!(d > 0.0)) *bad = 1;
      s[j][j] = sqrt(fmax(d, 1e-300));
    }
    __syncthreads();
    if (t > j && t < b) s[t][j] /= s[j][j];
    __syncthreads();
    if (t > j && t < b)
      for (int c = j + 1; c <= t; ++c) s[t][c] -= s[t][j] * s[c][j];
    __syncthreads();
  }
  if (t < b)
    for (int c = 0; c <= t; ++c) A[(size_t)(k + t) * ld + k + c] = s[t][c];
}

// Panel rows r >= k + b: L21[r, :] solves L11 L21[r, :]^T = A21[r, :]^T.
__global__ void k_trsm_panel(double* __restrict__ A, size_t ld, int n, int k, int b) {
  __shared__ double L[NB][NB + 1];
  for (int q = threadIdx.x; q < b * b; q += blockDim.x) {
    const int i = q / b, c = q % b;
    L[i][c] = c <= i ? A[(size_t)(k + i) * ld + k + c] : 0.0;
  }
  __syncthreads();
  const int r = k + b + blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  double* row = A + (size_t)r * ld + k;
  double l[NB];
  for (int j = 0; j < b; ++j) {
    double s = row[j];
    for (int m = 0; m < j; ++m) s -= l[m] * L[j][m];
    l[j] = s / L[j][j];
  }
  for (int j = 0; j < b; ++j) row[j] = l[j];
}

// Trailing update of the lower triangle: A22[i, j] -= sum_m L21[i, m] L21[j, m].
__global__ void __launch_bounds__(256) k_syrk_update(double* __restrict__ A, size_t ld, int n,
                                                     int k, int b) {
  const int ti = blockIdx.y, tj = blockIdx.x;
  if (tj > ti) return;
  const int r0 = k + b + ti * DTILE, c0 = k + b + tj * DTILE;
  __shared__ double Li[DTILE][NB + 1], Lj[DTILE][NB + 1];
  for (int q = threadIdx.x; q < DTILE * NB; q += blockDim.x) {
    const int rr = q / NB, m = q % NB;
    Li[rr][m] = (r0 + rr < n && m < b) ? A[(size_t)(r0 + rr) * ld + k + m] : 0.0;
    Lj[rr][m] = (c0 + rr < n && m < b) ? A[(size_t)(c0 + rr) * ld + k + m] : 0.0;
  }
  __syncthreads();
  const int ty = threadIdx.x / 16, tx = threadIdx.x % 16;  // 16 x 16 threads, 4 x 4 each
  double acc[4][4] = {};
  for (int m = 0; m < b; ++m) {
    double a[4], c[4];
    for (int u = 0; u < 4; ++u) {
      a[u] = Li[ty * 4 + u][m];
      c[u] = Lj[tx * 4 + u][m];
    }
    for (int u = 0; u < 4; ++u)
      for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], c[v], acc[u][v]);
  }
  for (int u = 0; u < 4; ++u)
    for (int v = 0; v < 4; ++v) {
      const int i = r0 + ty * 4 + u, j = c0 + tx * 4 + v;
      if (i < n && j < n && j <= i) A[(size_t)i * ld + j] -= acc[u][v];
    }
}

// Forward substitution, block kb: solve L[kb, kb] y_kb = rhs_kb (one CTA),
// then rhs[below] -= L[below, kb] y_kb.
__global__ void k_fwd_diag(const double* __restrict__ A, size_t ld, int k, int b,
                           double* __restrict__ y) {
  if (threadIdx.x != 0) return;
  for (int j = 0; j < b; ++j) {
    double s = y[k + j];
    for (int m = 0; m < j; ++m) s -= A[(size_t)(k + j) * ld + k + m] * y[k + m];
    y[k + j] = s / A[(size_t)(k + j) * ld + k + j];
  }
}

__global__ void k_fwd_update(const double* __restrict__ A, size_t ld, int n, int k, int b,
                             double* __restrict__ y) {
  const int r = k + b + blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  double s = 0.0;
  for (int m = 0; m < b; ++m) s = fma(A[(size_t)r * ld + k + m], y[k + m], s);
  y[r] -= s;
}

// Backward substitution with L^T, block kb (processed last to first).
__global__ void k_bwd_diag(const double* __restrict__ A, size_t ld, int k, int b,
                           double* __restrict__ x) {
  if (threadIdx.x != 0) return;
  for (int j = b - 1; j >= 0; --j) {
    double s = x[k + j];
    for (int m = j + 1; m < b; ++m) s -= A[(size_t)(k + m) * ld + k + j] * x[k + m];
    x[k + j] = s / A[(size_t)(k + j) * ld + k + j];
  }
}

__global__ void k_bwd_update(const double* __restrict__ A, size_t ld, int k, int b,
                             double* __restrict__ x) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;  // r < k
  if (r >= k) return;
  double s = 0.0;
  for (int m = 0; m < b; ++m) s = fma(A[(size_t)(k + m) * ld + r], x[k + m], s);
  x[r] -= s;
}

__global__ void k_scale(int n, const double* __restrict__ w, double* __restrict__ x) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] *= w[i];
}

// SoA coordinates and (wl, e, b) in caller order from the records.
__global__ void k_records_soa(int n, int form, const double* __restrict__ rec,
                             double* __restrict__ x, double* __restrict__ y,
                             double* __restrict__ z, double* __restrict__ wl,
                             double* __restrict__ e, double* __restrict__ b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* r = rec + (size_t)i * 5;
  x[i] = r[0];
  y[i] = r[1];
  z[i] = r[2];
  wl[i] = form == DS_FORM_W ? r[3] : 1.0;
  e[i] = form == DS_FORM_W ? 1.0 : r[3];
  b[i] = r[4];
}

}  // namespace

// ---- dense operator for PCG ------------------------------------------------

void op_free_dense(ds_operator* op) {
  op->dense.release();
  op->dense_vff.release();
  op->dense_part.release();
  op->dense_dot.release();
  op->dense_cnt.release();
}

void op_build_dense(ds_operator* op) {
  cudaStream_t st = op->ctx->stream;
  const size_t np = op->pix.n_pad;
  op->dense.alloc(np * np);
  DevBuf<unsigned long long> stats;
  stats.alloc(3);
  const unsigned long long init[3] = {~0ull, 0ull, 0ull};
  DS_CUDA(cudaMemcpyAsync(stats.p, init, sizeof(init), cudaMemcpyHostToDevice, st));
  const int sms = op->ctx->num_sms > 0 ? op->ctx->num_sms : 152;
  k_dense_build<<<std::min<size_t>(np, (size_t)sms * 8), 256, 0, st>>>(
      op->kc, (int)np, np, op->pix.x.p, op->pix.y.p, op->pix.z.p, op->wl.p, op->e.p,
      op->table.p, op->dense.p, stats.p);
  DS_CHECK_LAUNCH();
  unsigned long long h[3];
  DS_CUDA(cudaMemcpyAsync(h, stats.p, sizeof(h), cudaMemcpyDeviceToHost, st));
  DS_CUDA(cudaStreamSynchronize(st));
  const double lo = std::ldexp(1.0, -100), hi = std::ldexp(1.0, 100);
  double mn, mx;
  std::memcpy(&mn, &h[0], sizeof(double));
  std::memcpy(&mx, &h[1], sizeof(double));
  op->dense_ff_ok = mx <= hi && (h[0] == ~0ull || mn >= lo);
  op->dense_signed = h[2] != 0;
  const size_t nrb = np / DM_RB, ncb = (np + DM_CW - 1) / DM_CW;
  op->dense_vff.alloc(np);
  op->dense_part.alloc(ncb * np);
  op->dense_dot.alloc(nrb);
  op->dense_cnt.alloc(nrb + 1);
  DS_CUDA(cudaMemsetAsync(op->dense_cnt.p, 0, (nrb + 1) * sizeof(unsigned int), st));
}

int dense_arith_in_use(const ds_operator* op) {
  if (op->dense_arith == DS_DENSE_FP64 || !op->dense_ff_ok) return DS_DENSE_FP64;
  return DS_DENSE_FLOAT_PAIR;
}

namespace {

template <bool FF, bool SIGNED>
void launch_dense_mv(const DenseMv& a, bool residual, bool dot, int grid, cudaStream_t st) {
  constexpr int NT = DM_WARPS * 32;
  if (residual)
    k_dense_mv<FF, SIGNED, true, false><<<grid, NT, 0, st>>>(a);
  else if (dot)
    k_dense_mv<FF, SIGNED, false, true><<<grid, NT, 0, st>>>(a);
  else
    k_dense_mv<FF, SIGNED, false, false><<<grid, NT, 0, st>>>(a);
}

}  // namespace

void dense_apply(ds_operator* op, bool residual, const double* v, double* out,
                 const double* dotv, PcgState* pcg, const int* skip, cudaStream_t st) {
  const int np = op->pix.n_pad;
  require(np % DM_RB == 0 && op->dense.p, "dense operator not built");
  DenseMv a{};
  a.n = np;
  a.nrb = np / DM_RB;
  a.ncb = (np + DM_CW - 1) / DM_CW;
  a.A = op->dense.p;
  a.v = v;
  a.vff = op->dense_vff.p;
  a.b = op->b.p;
  a.out = out;
  a.dotv = dotv;
  a.part = op->dense_part.p;
  a.dot_part = op->dense_dot.p;
  a.rb_cnt = op->dense_cnt.p;
  a.cnt = op->dense_cnt.p + a.nrb;
  a.pcg = pcg;
  a.skip = skip;
  const bool ff = dense_arith_in_use(op) == DS_DENSE_FLOAT_PAIR;
  const int sms = op->ctx->num_sms > 0 ? op->ctx->num_sms : 152;
  const int grid = std::min(a.nrb * a.ncb, sms * DM_CTAS_PER_SM);
  Profiler& prof = op->ctx->prof;
  cudaEvent_t ev = nullptr;
  if (prof.enabled) {
    a.prof_pairs = prof.d_pairs + 3;
    prof.begin(st, &ev);
  }
  if (ff) {
    k_split_vec<<<std::min((np + 255) / 256, 4 * sms), 256, 0, st>>>(np, v, op->dense_vff.p,
                                                                    skip);
    DS_CHECK_LAUNCH();
    if (op->dense_signed)
      launch_dense_mv<true, true>(a, residual, dotv != nullptr, grid, st);
    else
      launch_dense_mv<true, false>(a, residual, dotv != nullptr, grid, st);
  } else {
    launch_dense_mv<false, true>(a, residual, dotv != nullptr, grid, st);
  }
  DS_CHECK_LAUNCH();
  if (ev) prof.end(st, ev, 3);
}

// ---- closed-form solve -------------------------------------------------------

void solve_cf_dev(ds_context* ctx, int form, int n, const double* d_rec,
                  const KernelConsts& kc, const double* d_table, double* d_x) {
  cudaStream_t st = ctx->stream;
  DevBuf<double> x, y, z, wl, e, A;
  x.alloc(n);
  y.alloc(n);
  z.alloc(n);
  wl.alloc(n);
  e.alloc(n);
  k_records_soa<<<(n + 255) / 256, 256, 0, st>>>(n, form, d_rec, x.p, y.p, z.p, wl.p, e.p, d_x);
  DS_CHECK_LAUNCH();
  A.alloc((size_t)n * n);
  k_dense_build<<<std::min(n, 152 * 8), 256, 0, st>>>(kc, n, n, x.p, y.p, z.p, wl.p, e.p, d_table,
                                                     A.p, nullptr);
  DS_CHECK_LAUNCH();
  DevBuf<int> bad;
  bad.alloc(1);
  DS_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), st));
  for (int k = 0; k < n; k += NB) {
    const int b = std::min(NB, n - k);
    k_potrf_diag<<<1, NB, 0, st>>>(A.p, n, k, b, bad.p);
    DS_CHECK_LAUNCH();
    const int rest = n - k - b;
    if (rest > 0) {
      k_trsm_panel<<<(rest + 127) / 128, 128, 0, st>>>(A.p, n, n, k, b);
      DS_CHECK_LAUNCH();
      const int nt = (rest + DTILE - 1) / DTILE;
      k_syrk_update<<<dim3(nt, nt), 256, 0, st>>>(A.p, n, n, k, b);
      DS_CHECK_LAUNCH();
    }
  }
  // L y = rhs (rhs in d_x), then L^T x = y.
  for (int k = 0; k < n; k += NB) {
    const int b = std::min(NB, n - k);
    k_fwd_diag<<<1, 32, 0, st>>>(A.p, n, k, b, d_x);
    DS_CHECK_LAUNCH();
    const int rest = n - k - b;
    if (rest > 0) {
      k_fwd_update<<<(rest + 127) / 128, 128, 0, st>>>(A.p, n, n, k, b, d_x);
      DS_CHECK_LAUNCH();
    }
  }
  for (int k = ((n - 1) / NB) * NB; k >= 0; k -= NB) {
    const int b = std::min(NB, n - k);
    k_bwd_diag<<<1, 32, 0, st>>>(A.p, n, k, b, d_x);
    DS_CHECK_LAUNCH();
    if (k > 0) {
      k_bwd_update<<<(k + 127) / 128, 128, 0, st>>>(A.p, n, k, b, d_x);
      DS_CHECK_LAUNCH();
    }
  }
  if (form == DS_FORM_W) {
    k_scale<<<(n + 255) / 256, 256, 0, st>>>(n, wl.p, d_x);
    DS_CHECK_LAUNCH();
  }
  int h_bad = 0;
  DS_CUDA(cudaMemcpyAsync(&h_bad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  DS_CUDA(cudaStreamSynchronize(st));
  require(!h_bad, "closed-form solve: the matrix is not positive definite");
}

}  // namespace ds
