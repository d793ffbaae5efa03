// Persistent form of the structured mixed-precision iteration (no reference
// counterpart; the recurrence is lib/pcg.h:27-160 with FP32 inner products
// and FP64-accurate reliable updates, exactly as in mixed.cu).
//
// The per-kernel iteration (mixed.cu) spends most of its time waiting: each
// of its kernels moves a few MB of L2-resident data in ~20 us, and the
// launch ramp, the chains of dependent loads and the single CTA that
// reduces the partials at the end of each kernel dominate.  Here one
// cooperative launch runs every iteration.  Each CTA owns whole blocks of the
// band preconditioner (a cluster of neighbouring skewers, or one skewer) and
// so every record of those skewers: only the structured product reads other
// CTAs' data (the neighbour skewers' z-convolution levels).  The CTAs pass
// through three phases per iteration, separated by grid-wide barriers, and
// each keeps its own copy of the CG scalars, computed from the same partials
// in the same order (so all copies agree bit for bit and nothing is
// broadcast):
//   A  p = z + beta p and the levels V^(L) of u = wr p, per owned skewer
//                                                          (barrier: V read)
//   B  q = A32 p and the partial p.q, per owned skewer     (barrier: alpha)
//   C  alpha = r.z / p.q; x += alpha p, r -= alpha q; z = G G^T r over each
//      owned block (in shared memory, no halo: G has no entry between
//      blocks); partials r.z, |r|^2; then beta and the update test
//                                                          (barrier: beta)
// and, when an FP64 update is due, D the FP64 levels of u = wr x (barrier),
// E r64 = b - A x and F r = r64, z = G G^T r with their partials (one CTA
// owns both, so no barrier between them; barrier).
// Data written by another CTA during the kernel is read through L2
// (ld.global.cg), never from a possibly stale L1 line.
//
// Every barrier wait is bounded (`limit` SM clock cycles): a CTA that runs
// out records the barrier's code, and every CTA leaves at its next barrier;
// the host reports DS_ERR_TIMEOUT.  The launch is cooperative (all CTAs
// resident), so a barrier always completes unless a CTA has left.
#include <algorithm>
#include <cmath>

#include "ds_device.cuh"
#include "ds_f32.h"
#include "ds_learned.h"
#include "ds_mixed_dev.cuh"
#include "ds_ops.h"
#include "ds_skewer.h"

namespace ds {
namespace {

constexpr int NT = 512;      // threads per CTA
constexpr int MAX_S = 1024;  // slots (records) per preconditioner block
constexpr int MAX_G = 8;     // skewers per block
constexpr int NB = 128;      // neighbour entries staged per skewer per round
constexpr int UF32 = 8;      // neighbour loads in flight per record: FP32 product
constexpr int UF64 = 4;      // FP64 product
constexpr int MAX_BAND = 32;
constexpr int RPT = MAX_S / NT;  // records (slots) per thread

struct PersistArgs {
  int n, n_per, n_blocks, S, g, band, max_iter;
  const int* bsk;   // block -> its g skewers (-1: none); null: block b = skewer b
  const int* crec;  // slot -> record (-1: padding); null: slot = record
  const float* L;   // band + 1 planes of n_blocks S slots
  // FP32 inner operator
  const int *iptr, *iidx, *ilev;
  const float *ip32, *taps32;
  int ilmax;
  float* V32;
  // FP64 outer operator
  const int *optr, *oidx, *olev;
  const double *op64, *taps64;
  int olmax;
  double* V64;
  // record-order coefficients and vectors
  const double *wl, *wr, *e, *b;
  double* x;
  float *p, *q, *r, *z;
  double* r64;
  // state and scratch
  MixedState* S_;
  double *hist, *htrue, *part;
  unsigned int *bar_count, *bar_gen;
  int* err;
  long long limit;
};

// Barrier codes: the phase whose closing barrier gave up.
enum { B_LEVELS = 1, B_PRODUCT, B_STEP, B_LEVELS64, B_UPDATE };

// Grid-wide barrier (all CTAs resident: cooperative launch).  Thread 0 reads
// the generation before arriving; the last to arrive resets the count and
// bumps the generation; the others poll it, bounded by `limit`.  Returns
// false when this CTA or another one has given up.
__device__ bool grid_sync(const PersistArgs& a, int code) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    volatile unsigned int* gen = a.bar_gen;
    volatile int* err = a.err;
    const unsigned int g = *gen;
    __threadfence();
    if (atomicAdd(a.bar_count, 1u) == gridDim.x - 1) {
      *(volatile unsigned int*)a.bar_count = 0;
      __threadfence();
      atomicAdd(a.bar_gen, 1u);
    } else {
      const long long t0 = clock64();
      while (*gen == g) {
        if (*err) {
          ok = 0;
          break;
        }
        if (clock64() - t0 > a.limit) {
          atomicExch(a.err, code);
          ok = 0;
          break;
        }
      }
    }
    __threadfence();
    ok_s = ok && *err == 0;
  }
  __syncthreads();
  return ok_s != 0;
}

// Sum of n partials (stride, offset) in a fixed order, valid in every thread
// of every CTA alike.
__device__ __forceinline__ double partial_total(const double* part, int n, int stride, int off,
                                                double* red, double* out) {
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += NT) v += __ldcg(part + (size_t)i * stride + off);
  const double s = block_sum<NT>(v, red);
  if (threadIdx.x == 0) *out = s;
  __syncthreads();
  const double t = *out;
  __syncthreads();
  return t;
}

__device__ __forceinline__ int skewer_of(const PersistArgs& a, int blk, int j) {
  return a.bsk ? a.bsk[(size_t)blk * a.g + j] : (j == 0 ? blk : -1);
}

__device__ __forceinline__ int record_of(const PersistArgs& a, int blk, int i) {
  const size_t slot = (size_t)blk * a.S + i;
  return a.crec ? a.crec[slot] : (int)slot;
}

// Levels V^(L)[k] = sum_{|m| <= L} T_m u[k + m] (L = 0 .. lmax) of every
// skewer of block blk, u = ufn(record) staged in shared memory (g n_per).
template <typename T, class UFn>
__device__ __forceinline__ void block_levels(const PersistArgs& a, int blk, int lmax,
                                             const T* __restrict__ taps, T* __restrict__ V,
                                             T* su, UFn&& ufn) {
  const int m = a.g * a.n_per;
  const size_t n = (size_t)a.n;
  __syncthreads();
  for (int i = threadIdx.x; i < m; i += NT) {
    const int j = i / a.n_per, k = i - j * a.n_per;
    const int s = skewer_of(a, blk, j);
    su[i] = s >= 0 ? ufn((size_t)s * a.n_per + k) : T(0);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < m; i += NT) {
    const int j = i / a.n_per, k = i - j * a.n_per;
    const int s = skewer_of(a, blk, j);
    if (s < 0) continue;
    const size_t r = (size_t)s * a.n_per + k;
    T acc = su[i];
    V[r] = acc;
    for (int l = 1; l <= lmax; ++l) {
      T v = T(0);
      if (k + l < a.n_per) v = su[i + l];
      if (k - l >= 0) v += su[i - l];
      acc = fma(taps[l], v, acc);
      V[(size_t)l * n + r] = acc;
    }
  }
}

// out[t] = sum over the neighbour list of the skewer of record t of
// P V[(lev - 1) n + idx n_per + k], for the (up to RPT) records t = tid,
// tid + NT, ... of block blk (record t: pixel k of the block's skewer j,
// t = j n_per + k): the g lists are staged NB entries at a time; each step
// keeps UF loads per record in flight.
template <typename T, int UF>
__device__ __forceinline__ void block_product(const PersistArgs& a, int blk,
                                              const int* __restrict__ ptr,
                                              const int* __restrict__ idx,
                                              const int* __restrict__ lev,
                                              const T* __restrict__ pv, const T* V,
                                              size_t* s_off, T* s_p, int* s_cnt, T (&out)[RPT]) {
  const int m = a.g * a.n_per;
  const size_t n = (size_t)a.n;
  T acc[RPT][UF];
#pragma unroll
  for (int t = 0; t < RPT; ++t)
#pragma unroll
    for (int u = 0; u < UF; ++u) acc[t][u] = T(0);
  int jj[RPT], kk[RPT];
#pragma unroll
  for (int t = 0; t < RPT; ++t) {
    const int i = threadIdx.x + t * NT;
    jj[t] = i < m ? i / a.n_per : -1;
    kk[t] = i < m ? i - jj[t] * a.n_per : 0;
  }
  for (int c0 = 0;; c0 += NB) {
    __syncthreads();
    if (threadIdx.x < MAX_G) {
      const int j = threadIdx.x;
      const int s = j < a.g ? skewer_of(a, blk, j) : -1;
      const int len = s >= 0 ? ptr[s + 1] - ptr[s] : 0;
      s_cnt[j] = max(0, min(NB, len - c0));
      s_cnt[MAX_G + j] = len - c0 > NB;  // another round
    }
    for (int t = threadIdx.x; t < a.g * NB; t += NT) {
      const int j = t / NB, e = t - j * NB;
      const int s = skewer_of(a, blk, j);
      if (s < 0) continue;
      const int q = ptr[s] + c0 + e;
      if (q < ptr[s + 1]) {
        s_off[t] = (size_t)(lev[q] - 1) * n + (size_t)idx[q] * a.n_per;
        s_p[t] = pv[q];
      }
    }
    __syncthreads();
    int cnt[RPT];
#pragma unroll
    for (int t = 0; t < RPT; ++t) cnt[t] = jj[t] >= 0 ? s_cnt[jj[t]] : 0;
    int cmax = 0;
#pragma unroll
    for (int t = 0; t < RPT; ++t) cmax = max(cmax, cnt[t]);
    for (int e = 0; e < cmax; e += UF) {
      T v[RPT][UF];
#pragma unroll
      for (int t = 0; t < RPT; ++t)
#pragma unroll
        for (int u = 0; u < UF; ++u)
          v[t][u] = e + u < cnt[t] ? __ldcg(V + s_off[jj[t] * NB + e + u] + kk[t]) : T(0);
#pragma unroll
      for (int t = 0; t < RPT; ++t)
#pragma unroll
        for (int u = 0; u < UF; ++u)
          if (e + u < cnt[t]) acc[t][u] = fma(s_p[jj[t] * NB + e + u], v[t][u], acc[t][u]);
    }
    int more = 0;
    for (int j = 0; j < MAX_G; ++j) more |= s_cnt[MAX_G + j];
    if (!more) break;
  }
#pragma unroll
  for (int t = 0; t < RPT; ++t) {
    T s = T(0);
#pragma unroll
    for (int u = 0; u < UF; ++u) s += acc[t][u];
    out[t] = s;
  }
}

// z = G G^T r over block blk from r in shared memory (slot order, 0 on
// padding): t = G^T r, then z = G t; returns z of the thread's slots.
template <int BAND>
__device__ __forceinline__ void block_precond(const PersistArgs& a, int blk, const float* rs,
                                              float* ts, float (&zk)[RPT]) {
  const int band = BAND >= 0 ? BAND : a.band;
  const size_t ns = (size_t)a.n_blocks * a.S;
  const size_t s0 = (size_t)blk * a.S;
  const float* __restrict__ L = a.L;
#pragma unroll
  for (int t = 0; t < RPT; ++t) {
    const int i = threadIdx.x + t * NT;
    if (i < a.S) {
      float v = 0.f;
#pragma unroll
      for (int m = 0; m <= (BAND >= 0 ? BAND : MAX_BAND); ++m)
        if (m <= band && i + m < a.S) v = fmaf(L[(size_t)m * ns + s0 + i + m], rs[i + m], v);
      ts[i] = v;
    }
  }
  __syncthreads();
#pragma unroll
  for (int t = 0; t < RPT; ++t) {
    const int i = threadIdx.x + t * NT;
    float v = 0.f;
    if (i < a.S) {
#pragma unroll
      for (int m = 0; m <= (BAND >= 0 ? BAND : MAX_BAND); ++m)
        if (m <= band && i - m >= 0) v = fmaf(L[(size_t)m * ns + s0 + i], ts[i - m], v);
    }
    zk[t] = v;
  }
}

template <int BAND>
__global__ void __launch_bounds__(NT, 2) k_mixed_persistent(PersistArgs a) {
  __shared__ MixedState sS;
  __shared__ double red[NT / 32];
  __shared__ double tot;
  __shared__ __align__(16) double su64[MAX_S];  // u of a block (FP64 or FP32)
  __shared__ float rs[MAX_S];
  __shared__ float ts[MAX_S];
  __shared__ size_t s_off[MAX_G * NB];
  __shared__ double s_p64[MAX_G * NB];
  __shared__ int s_cnt[2 * MAX_G];
  float* su = reinterpret_cast<float*>(su64);
  float* s_p32 = reinterpret_cast<float*>(s_p64);
  const int tid = threadIdx.x;
  const int G = gridDim.x;
  if (tid == 0) sS = *a.S_;
  __syncthreads();
  // the recurrence sets done by iteration max_iter at the latest (the
  // update it forces there ends the solve); the bound keeps hist in range
  while (!sS.done && sS.iter < a.max_iter) {
    const int it = sS.iter + 1;
    // ---- A: p = z + beta p, levels of u = wr p
    {
      const float beta = (float)sS.beta;
      for (int blk = blockIdx.x; blk < a.n_blocks; blk += G)
        block_levels<float>(a, blk, a.ilmax, a.taps32, a.V32, su, [&](size_t r) {
          const float pv = fmaf(beta, __ldcg(a.p + r), __ldcg(a.z + r));
          a.p[r] = pv;
          return (float)a.wr[r] * pv;
        });
    }
    if (!grid_sync(a, B_LEVELS)) break;
    // ---- B: q = A32 p, partial p.q
    double dq = 0.0;
    for (int blk = blockIdx.x; blk < a.n_blocks; blk += G) {
      float acc[RPT];
      block_product<float, UF32>(a, blk, a.iptr, a.iidx, a.ilev, a.ip32, a.V32, s_off, s_p32, s_cnt,
                           acc);
#pragma unroll
      for (int t = 0; t < RPT; ++t) {
        const int i = tid + t * NT;
        if (i >= a.g * a.n_per) continue;
        const int j = i / a.n_per;
        const int s = skewer_of(a, blk, j);
        if (s < 0) continue;
        const size_t r = (size_t)s * a.n_per + (i - j * a.n_per);
        const float pv = __ldcg(a.p + r);
        const float qv = fmaf((float)a.wl[r], acc[t], (float)a.e[r] * pv);
        a.q[r] = qv;
        dq = fma((double)pv, (double)qv, dq);
      }
    }
    {
      const double bs = block_sum<NT>(dq, red);
      if (tid == 0) a.part[blockIdx.x] = bs;
    }
    if (!grid_sync(a, B_PRODUCT)) break;
    // ---- C: alpha; x, r, z per owned block; partials r.z, |r|^2
    const double pq = partial_total(a.part, G, 1, 0, red, &tot);
    const double alpha_d = sS.rz / pq;
    const float alpha = (float)alpha_d;
    double rz = 0.0, rr = 0.0;
    for (int blk = blockIdx.x; blk < a.n_blocks; blk += G) {
      __syncthreads();  // rs, ts of the previous block read
      int rec[RPT];
#pragma unroll
      for (int t = 0; t < RPT; ++t) {
        const int i = tid + t * NT;
        rec[t] = i < a.S ? record_of(a, blk, i) : -1;
        if (i < a.S) {
          float rv = 0.f;
          if (rec[t] >= 0) {
            const int k = rec[t];
            rv = fmaf(-alpha, __ldcg(a.q + k), __ldcg(a.r + k));
            a.x[k] = fma(alpha_d, (double)__ldcg(a.p + k), __ldcg(a.x + k));
            a.r[k] = rv;
          }
          rs[i] = rv;
        }
      }
      __syncthreads();
      float zk[RPT];
      block_precond<BAND>(a, blk, rs, ts, zk);
#pragma unroll
      for (int t = 0; t < RPT; ++t) {
        if (rec[t] < 0) continue;
        const float ri = rs[tid + t * NT];
        a.z[rec[t]] = zk[t];
        rz = fma((double)ri, (double)zk[t], rz);
        rr = fma((double)ri, (double)ri, rr);
      }
    }
    {
      const double b1 = block_sum<NT>(rz, red);
      const double b2 = block_sum<NT>(rr, red);
      if (tid == 0) {
        a.part[(size_t)G + 2 * blockIdx.x] = b1;
        a.part[(size_t)G + 2 * blockIdx.x + 1] = b2;
      }
    }
    if (!grid_sync(a, B_STEP)) break;
    // the step's scalars (those of K2 in the per-kernel form), every CTA alike
    {
      const double trz = partial_total(a.part + G, G, 2, 0, red, &tot);
      const double trr = partial_total(a.part + G, G, 2, 1, red, &tot);
      if (tid == 0) {
        sS.alpha = alpha_d;
        sS.pq = pq;
        sS.rz_old = sS.rz;
        sS.rz = trz;
        sS.rnorm = sqrt(trr);
        sS.iter = it;
        if (blockIdx.x == 0) a.hist[it] = sS.rnorm;
        sS.rmax = fmax(sS.rmax, sS.rnorm);
        sS.need_update = update_due(&sS, it) ? 1 : 0;
        sS.beta = sS.rz / sS.rz_old;
      }
      __syncthreads();
    }
    if (!sS.need_update) continue;
    // ---- D: FP64 levels of u = wr x
    for (int blk = blockIdx.x; blk < a.n_blocks; blk += G)
      block_levels<double>(a, blk, a.olmax, a.taps64, a.V64, su64,
                           [&](size_t r) { return a.wr[r] * __ldcg(a.x + r); });
    if (!grid_sync(a, B_LEVELS64)) break;
    // ---- E, F: r64 = b - A x per owned skewer; r = r64, z = G G^T r
    rz = 0.0;
    rr = 0.0;
    for (int blk = blockIdx.x; blk < a.n_blocks; blk += G) {
      double acc[RPT];
      block_product<double, UF64>(a, blk, a.optr, a.oidx, a.olev, a.op64, a.V64, s_off, s_p64, s_cnt,
                            acc);
#pragma unroll
      for (int t = 0; t < RPT; ++t) {
        const int i = tid + t * NT;
        if (i >= a.g * a.n_per) continue;
        const int j = i / a.n_per;
        const int s = skewer_of(a, blk, j);
        if (s < 0) continue;
        const size_t r = (size_t)s * a.n_per + (i - j * a.n_per);
        const double y = fma(a.wl[r], acc[t], a.e[r] * __ldcg(a.x + r));
        a.r64[r] = a.b[r] - y;
      }
      __syncthreads();  // the block's r64 written (read below in slot order)
      int rec[RPT];
#pragma unroll
      for (int t = 0; t < RPT; ++t) {
        const int i = tid + t * NT;
        rec[t] = i < a.S ? record_of(a, blk, i) : -1;
        if (i < a.S) {
          float rv = 0.f;
          if (rec[t] >= 0) {
            const double rd = __ldcg(a.r64 + rec[t]);
            rv = (float)rd;
            a.r[rec[t]] = rv;
            rr = fma(rd, rd, rr);
          }
          rs[i] = rv;
        }
      }
      __syncthreads();
      float zk[RPT];
      block_precond<BAND>(a, blk, rs, ts, zk);
#pragma unroll
      for (int t = 0; t < RPT; ++t) {
        if (rec[t] < 0) continue;
        a.z[rec[t]] = zk[t];
        rz = fma((double)rs[tid + t * NT], (double)zk[t], rz);
      }
    }
    {
      const double b1 = block_sum<NT>(rz, red);
      const double b2 = block_sum<NT>(rr, red);
      if (tid == 0) {
        a.part[(size_t)G + 2 * blockIdx.x] = b1;
        a.part[(size_t)G + 2 * blockIdx.x + 1] = b2;
      }
    }
    if (!grid_sync(a, B_UPDATE)) break;
    // the update's scalars (those of K6), every CTA alike
    {
      const double trz = partial_total(a.part + G, G, 2, 0, red, &tot);
      const double trr = partial_total(a.part + G, G, 2, 1, red, &tot);
      if (tid == 0) {
        const double rt = sqrt(trr);
        sS.rtrue = rt;
        ++sS.n_updates;
        if (blockIdx.x == 0) {
          a.htrue[sS.n_updates] = rt;
          a.hist[sS.iter] = rt;
        }
        if (rt <= sS.tol_norm_b) {
          sS.done = 1;
          sS.converged = 1;
        } else if (sS.iter >= sS.max_iter) {
          sS.done = 1;
        } else {
          sS.rz = trz;
          restart_after_update(&sS, rt, trz);
        }
        sS.need_update = 0;
      }
      __syncthreads();
    }
  }
  if (blockIdx.x == 0 && tid == 0) {
    sS.skip_update = 1;
    *a.S_ = sS;
  }
}

// CTAs of the cooperative launch: one per block, at most the resident count.
template <int BAND>
int persistent_grid(int num_sms, int n_blocks) {
  static int per_sm = -1;
  if (per_sm < 0) {
    DS_CUDA(cudaFuncSetAttribute(k_mixed_persistent<BAND>,
                                 cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared));
    DS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mixed_persistent<BAND>, NT,
                                                          0));
  }
  return std::min(per_sm * num_sms, n_blocks);
}

}  // namespace

bool run_mixed_persistent(ds_operator* op, OpF32& f, const SkewerPC* pc, const SkewerVecs& sv,
                          double* X, float* r, int max_iter, cudaStream_t st) {
  SkewerGrid& g = *op->sgrid;
  if (!pc || pc->band > MAX_BAND || pc->g > MAX_G || pc->n_per > MAX_S || pc->n_sk <= 0)
    return false;
  // blocks of whole skewers of the grid: g skewers of n_per records each
  if (pc->n_per != pc->g * g.n_per || (pc->g > 1 && !pc->bsk.p) ||
      (long long)pc->n_sk * pc->g < g.n_sk)
    return false;
  if (!g.inner.ptr.p || !g.V32.p || !g.V64.p) return false;
  const int band = pc->band;
  const int grid = band == 16  ? persistent_grid<16>(op->ctx->num_sms, pc->n_sk)
                   : band == 2 ? persistent_grid<2>(op->ctx->num_sms, pc->n_sk)
                               : persistent_grid<-1>(op->ctx->num_sms, pc->n_sk);
  if (grid <= 0) return false;
  g.p_part.alloc((size_t)3 * grid);
  g.p_sync.alloc(3);
  DS_CUDA(cudaMemsetAsync(g.p_sync.p, 0, 3 * sizeof(int), st));
  PersistArgs a{};
  a.n = op->n;
  a.n_per = g.n_per;
  a.n_blocks = pc->n_sk;
  a.S = pc->n_per;
  a.g = pc->g;
  a.band = band;
  a.max_iter = max_iter;
  a.bsk = pc->bsk.p;  // null: the learned per-skewer factor (block b = skewer b)
  a.crec = pc->crec.p;
  a.L = pc->L.p;
  a.iptr = g.inner.ptr.p;
  a.iidx = g.inner.idx.p;
  a.ilev = g.inner.lev.p;
  a.ip32 = g.inner.p32.p;
  a.taps32 = g.taps32.p;
  a.ilmax = g.inner.lmax;
  a.V32 = g.V32.p;
  a.optr = g.outer.ptr.p;
  a.oidx = g.outer.idx.p;
  a.olev = g.outer.lev.p;
  a.op64 = g.outer.p64.p;
  a.taps64 = g.taps64.p;
  a.olmax = g.outer.lmax;
  a.V64 = g.V64.p;
  a.wl = sv.wl;
  a.wr = sv.wr;
  a.e = sv.e;
  a.b = sv.b;
  a.x = X;
  a.p = f.p.p;
  a.q = f.q.p;
  a.r = r;
  a.z = f.z.p;
  a.r64 = op->r.p;
  a.S_ = f.state.p;
  a.hist = f.hist.p;
  a.htrue = f.htrue.p;
  a.part = g.p_part.p;
  a.bar_count = reinterpret_cast<unsigned int*>(g.p_sync.p);
  a.bar_gen = reinterpret_cast<unsigned int*>(g.p_sync.p) + 1;
  a.err = g.p_sync.p + 2;
  a.limit = op->ctx->wait_limit > 0 ? op->ctx->wait_limit : 4000000000LL;
  void* args[] = {&a};
  const void* fn = band == 16  ? (const void*)k_mixed_persistent<16>
                   : band == 2 ? (const void*)k_mixed_persistent<2>
                               : (const void*)k_mixed_persistent<-1>;
  DS_CUDA(cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(NT), args, 0, st));
  DS_CHECK_LAUNCH();
  return true;
}

int persistent_error(ds_operator* op, cudaStream_t st) {
  SkewerGrid& g = *op->sgrid;
  if (!g.p_sync.p) return 0;
  int code = 0;
  DS_CUDA(cudaMemcpyAsync(&code, g.p_sync.p + 2, sizeof(int), cudaMemcpyDeviceToHost, st));
  DS_CUDA(cudaStreamSynchronize(st));
  if (code) DS_CUDA(cudaMemsetAsync(g.p_sync.p, 0, 3 * sizeof(int), st));
  return code;
}

}  // namespace ds
