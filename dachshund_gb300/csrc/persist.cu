// Persistent form of the structured mixed-precision iteration (no reference
// counterpart; the recurrence is lib/pcg.h:27-160 with FP32 inner products
// and FP64-accurate reliable updates, as in mixed.cu).
//
// The per-kernel iteration (mixed.cu) spends most of its time waiting: each
// of its kernels moves a few MB of L2-resident data in ~20 us, and the
// launch ramp, the chains of dependent loads, the single CTA that reduces
// the partials at the end of each kernel and the FP64 arithmetic of the
// iterate and the dot products (GB300 issues FP64 at 1/64 of FP32)
// dominate.  Here one cooperative launch runs every iteration.  Each CTA
// owns whole blocks of the band preconditioner (a cluster of neighbouring
// skewers, or one skewer) and so every record of those skewers: only the
// structured product reads other CTAs' data (the neighbour skewers'
// z-convolution levels).  Every CTA keeps its own copy of the CG scalars,
// computed from the same partials in the same order (so all copies agree bit
// for bit and nothing is broadcast).
//
// Two forms:
//  * k_mixed_resident (one block per CTA, every CTA resident): the block's
//    vectors, product items and FP16 factor stay in shared memory; two
//    phases per iteration (Chronopoulos and Gear's arrangement of the same
//    recurrence):
//      product  w = A32 z from the published levels of z (each distinct
//               (neighbour, level) row of the cluster loaded once; the rows
//               of its own skewers while the previous barrier completes),
//               p = z + beta p, q = w + beta q (= A32 p), the partial
//               p.q                                                   (barrier)
//      step     alpha; x += alpha p (float pairs), r -= alpha q, z = G G^T r
//               over the block (no halo: G has no entry between blocks), the
//               levels of z, the partials r.z, |r|^2; beta and the update
//               test                                                  (barrier)
//    and, when a reliable update is due, the float-pair levels of x (barrier)
//    and b - A x in float pairs, r, z and its levels (barrier).
//  * k_mixed_persistent (any number of blocks per CTA): the vectors in
//    global memory, three phases per iteration (p = z + beta p and the
//    levels of p; q = A32 p; alpha and the step), FP64 iterate.
// Data written by another CTA during the kernel is read through L2
// (ld.global.cg), never from a possibly stale L1 line.
//
// Every barrier wait is bounded (`limit` SM clock cycles): a CTA that runs
// out records the barrier's code, and every CTA leaves when it finds the
// code (in that barrier's wait or the next); the host reports
// DS_ERR_TIMEOUT.  The launch is cooperative (all CTAs
// resident), so a barrier always completes unless a CTA has left.  Phase
// timers (%globaltimer) accumulate per launch for the profile.
#include <algorithm>
#include <cmath>
#include <vector>

#include <cuda_fp16.h>

#include "ds_device.cuh"
#include "ds_ff.cuh"
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
constexpr int NB = 128;      // neighbour entries staged per skewer per round (general form)
constexpr int NB_R = 32;     // the same for the resident form's FP64 residual
constexpr int UF32 = 8;      // neighbour loads in flight per record: FP32 product
constexpr int UF64 = 4;      // FP64 product
constexpr int UFI = 16;      // FP32 product of the resident form: neighbour rows in flight
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
  unsigned int* bar;  // barrier words: count, error code
  int* err;
  long long limit;
  unsigned long long* pt;  // phase timers (PT_* layout)
  // the resident form's product items, NI slots per block (it_cnt: the
  // count of each block; an item is one (neighbour skewer, level) row: its
  // offset into the levels and the factor for each of the block's (<= 4)
  // skewers, 0 where unused)
  const int* it_cnt;
  const int* it_own;  // per block: its items on the block's own skewers (the first ones)
  const unsigned int* it_off;
  const float4* it_coef;
  // float-pair copies for the resident form's update (record order; the
  // outer lists' factors; the z taps)
  const float2 *wl_ff, *wr_ff, *e_ff, *b_ff, *op_ff, *taps64_ff;
};

// Barrier codes: the phase whose closing barrier gave up (also the phase
// timers' index); B_CALIB: the empty barrier after the start that
// calibrates the barrier's own cost (the profile's barrier_us).  Measured on
// GB300: without it the same solve ran ~20% slower (every iteration, not only
// the first; a code-generation effect whose cause is not known), with 1 to
// 16 of them the time is the same to 1%.
enum { B_LEVELS = 1, B_PRODUCT, B_STEP, B_LEVELS64, B_UPDATE, B_CALIB };
constexpr int N_CALIB = 1;

// Phase timers (%globaltimer, ns), accumulated over launches until read:
// CTA 0 records, per barrier code, the time from the previous barrier's exit
// to this one's exit and the number of visits; every CTA records, per code,
// its own work (from its previous exit to its arrival), so the slowest CTA
// and the barrier's wait are told apart.
enum {
  PT_LAST = 0,       // CTA 0's last exit
  PT_PHASE = 0,      // + code: exit-to-exit totals (codes 1..6)
  PT_VISITS = 8,     // + code
  PT_START = 16,     // kernel start (CTA 0)
  PT_KERNEL = 17,    // kernel time
  PT_LAUNCHES = 18,
  PT_GRID = 19,
  PT_CTA = 32        // + 8 blk + code: CTA work
};
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Grid-wide barrier (all CTAs resident: cooperative launch).  Every CTA's
// thread 0 arrives on one monotonic count (atom.acq_rel: it releases the
// CTA's writes, ordered before it by the CTA barrier) and polls the same
// count (ld.acquire) until it reaches epoch x CTAs: reading the last
// arrival's value synchronises with every arrival (the arrivals form one
// release sequence), and the CTA whose arrival completes the epoch does not
// poll at all.  (Measured on GB300 against a broadcast in which that CTA
// writes the epoch into a flag line per CTA after a fence: 2.90 against
// 3.07 ms per 262,144-pixel solve; the broadcast adds a fence and a store
// round trip to every barrier.)  A wait that runs out (`limit` SM cycles,
// checked before each poll) records `code` in the error word and returns
// false, as does a CTA that finds the error word set (read every 16 polls,
// and by the last arrival).
// Words: [0] count, [1] error code.
// The barrier comes in two halves: between grid_arrive and grid_wait a CTA
// may work on its own data (writing nothing another CTA reads in the next
// phase), which hides that work behind the barrier's latency.
constexpr int BAR_WORDS = 32;  // one 128-byte line
struct BarState {                  // thread 0's barrier state
  unsigned int epoch = 0;          // barriers passed
  unsigned long long exit_ns = 0;  // last exit (%globaltimer)
  int last = 0;                    // this CTA completed the current epoch
};

__device__ void grid_arrive(const PersistArgs& a, int code, BarState& b) {
  __syncthreads();
  if (threadIdx.x == 0) {
    if (b.epoch > 0) a.pt[PT_CTA + 8 * blockIdx.x + code] += global_ns() - b.exit_ns;
    ++b.epoch;
    const unsigned int target = b.epoch * gridDim.x;
    unsigned int old;
    asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], 1;"
                 : "=r"(old)
                 : "l"(a.bar)
                 : "memory");
    b.last = old + 1 == target;
  }
}

__device__ bool grid_wait(const PersistArgs& a, int code, BarState& b) {
  __shared__ int ok_s;
  if (threadIdx.x == 0) {
    int ok = 1;
    if (!b.last) {
      const unsigned int target = b.epoch * gridDim.x;
      const long long t0 = clock64();
      for (int k = 0;; ++k) {
        // the bound first: a CTA gives up once it has waited `limit`
        // cycles, whatever its next poll would read
        if (clock64() - t0 >= a.limit) {
          atomicExch(a.err, code);
          ok = 0;
          break;
        }
        unsigned int f;
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(f) : "l"(a.bar) : "memory");
        if ((int)(f - target) >= 0) break;
        if ((k & 15) == 15 && *(volatile int*)a.err) {
          ok = 0;
          break;
        }
      }
    } else if (*(volatile int*)a.err) {
      ok = 0;
    }
    const unsigned long long now = global_ns();
    b.exit_ns = now;
    if (blockIdx.x == 0) {
      a.pt[PT_PHASE + code] += now - a.pt[PT_LAST];
      a.pt[PT_LAST] = now;
      a.pt[PT_VISITS + code] += 1;
    }
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

__device__ __forceinline__ bool grid_sync(const PersistArgs& a, int code, BarState& b) {
  grid_arrive(a, code, b);
  return grid_wait(a, code, b);
}

// Sum of n partials in a fixed order, valid in every thread of every CTA
// alike: warp 0 alone sums them in FP64 (lane l takes l, l + 32, ..., then a
// shuffle tree), so the FP64 pipe (2 operations per clock per SM on GB300)
// sees n + 5 additions per CTA instead of a CTA-wide tree.
__device__ __forceinline__ double partial_total(const double* part, int n, double* out) {
  if (threadIdx.x < 32) {
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += 32) v += __ldcg(part + i);
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) *out = v;
  }
  __syncthreads();
  const double t = *out;
  __syncthreads();
  return t;
}

// The same for n pairs of partials (both sums from one pass over them).
__device__ __forceinline__ double2 partial_total2(const double* part, int n, double* out) {
  if (threadIdx.x < 32) {
    double v0 = 0.0, v1 = 0.0;
    for (int i = threadIdx.x; i < n; i += 32) {
      const double2 pr = __ldcg(reinterpret_cast<const double2*>(part) + i);
      v0 += pr.x;
      v1 += pr.y;
    }
    for (int o = 16; o > 0; o >>= 1) {
      v0 += __shfl_down_sync(0xffffffffu, v0, o);
      v1 += __shfl_down_sync(0xffffffffu, v1, o);
    }
    if (threadIdx.x == 0) {
      out[0] = v0;
      out[1] = v1;
    }
  }
  __syncthreads();
  const double2 t = make_double2(out[0], out[1]);
  __syncthreads();
  return t;
}

// Sum over the CTA of one float pair per thread (fixed order: a float-pair
// shuffle tree within each warp, then the warps' sums in FP64 by thread 0,
// where the result is valid).  The FP32 Krylov vectors' dot products are
// summed this way: exact products (FMA) and compensated sums keep about 44
// bits, and the FP64 pipe sees NT/32 additions per CTA.
__device__ __forceinline__ double block_sum_ff(ff v, double* sm /* NT/32 */) {
  for (int o = 16; o > 0; o >>= 1) {
    ff w;
    w.h = __shfl_down_sync(0xffffffffu, v.h, o);
    w.l = __shfl_down_sync(0xffffffffu, v.l, o);
    v = ff_add(v, w);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sm[wid] = (double)v.h + (double)v.l;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < NT / 32; ++w) s += sm[w];
  return s;
}

// a += x y exactly rounded to a float pair (the product's error by FMA).
__device__ __forceinline__ void ff_acc_prod(ff& a, float x, float y) {
  ff p;
  p.h = __fmul_rn(x, y);
  p.l = __fmaf_rn(x, y, -p.h);
  a = ff_add(a, p);
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
template <typename T, int UF, int NB>
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
// padding): t = G^T r, then z = G t; returns z of the thread's slots.  The
// factor's plane m, slot i of the block is L[m ls + i] (the CTA's copy in
// shared memory, or the global planes).
template <int BAND>
__device__ __forceinline__ void block_precond(const PersistArgs& a, const float* L, size_t ls,
                                              const float* rs, float* ts, float (&zk)[RPT]) {
  const int band = BAND >= 0 ? BAND : a.band;
  const size_t ns = ls;
  const size_t s0 = 0;
#pragma unroll
  for (int t = 0; t < RPT; ++t) {
    const int i = threadIdx.x + t * NT;
    if (i < a.S) {
      float v = 0.f;
#pragma unroll(BAND >= 0 ? BAND + 1 : 1)
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
#pragma unroll(BAND >= 0 ? BAND + 1 : 1)
      for (int m = 0; m <= (BAND >= 0 ? BAND : MAX_BAND); ++m)
        if (m <= band && i - m >= 0) v = fmaf(L[(size_t)m * ns + s0 + i], ts[i - m], v);
    }
    zk[t] = v;
  }
}

// The step's scalars (those of K2 in the per-kernel form), thread 0 of every
// CTA alike; CTA 0 records the history.
__device__ __forceinline__ void step_scalars(MixedState& sS, const PersistArgs& a, int it,
                                             double alpha_d, double pq, double trz, double trr) {
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

// The update's scalars (those of K6), thread 0 of every CTA alike.
__device__ __forceinline__ void update_scalars(MixedState& sS, const PersistArgs& a, double trz,
                                               double trr) {
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

// ---- general form: any number of blocks per CTA, vectors in global memory
template <int BAND>
__global__ void __launch_bounds__(NT, 2) k_mixed_persistent(PersistArgs a) {
  __shared__ MixedState sS;
  __shared__ double red[NT / 32];
  __shared__ double tot[2];
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
  const int P2 = (G + 1) & ~1;  // the pair partials start 16-byte aligned
  const size_t ns = (size_t)a.n_blocks * a.S;
  BarState bst;  // barrier state (thread 0)
  if (tid == 0) sS = *a.S_;
  if (tid == 0 && blockIdx.x == 0) {
    const unsigned long long now = global_ns();
    a.pt[PT_LAST] = now;
    a.pt[PT_START] = now;
    a.pt[PT_GRID] = gridDim.x;
    a.pt[PT_LAUNCHES] += 1;
  }
  __syncthreads();
  for (int k = 0; k < N_CALIB; ++k) grid_sync(a, B_CALIB, bst);
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
    if (!grid_sync(a, B_LEVELS, bst)) break;
    // ---- B: q = A32 p, partial p.q
    double dq = 0.0;
    for (int blk = blockIdx.x; blk < a.n_blocks; blk += G) {
      float acc[RPT];
      block_product<float, UF32, NB>(a, blk, a.iptr, a.iidx, a.ilev, a.ip32, a.V32, s_off, s_p32,
                                 s_cnt, acc);
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
    if (!grid_sync(a, B_PRODUCT, bst)) break;
    // ---- C: alpha; x, r, z per owned block; partials r.z, |r|^2
    const double pq = partial_total(a.part, G, tot);
    if (tid == 0) tot[0] = sS.rz / pq;
    __syncthreads();
    const double alpha_d = tot[0];
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
      block_precond<BAND>(a, a.L + (size_t)blk * a.S, ns, rs, ts, zk);
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
        a.part[(size_t)P2 + 2 * blockIdx.x] = b1;
        a.part[(size_t)P2 + 2 * blockIdx.x + 1] = b2;
      }
    }
    if (!grid_sync(a, B_STEP, bst)) break;
    {
      const double2 t2 = partial_total2(a.part + P2, G, tot);
      if (tid == 0) step_scalars(sS, a, it, alpha_d, pq, t2.x, t2.y);
      __syncthreads();
    }
    if (!sS.need_update) continue;
    // ---- D: FP64 levels of u = wr x
    for (int blk = blockIdx.x; blk < a.n_blocks; blk += G)
      block_levels<double>(a, blk, a.olmax, a.taps64, a.V64, su64,
                           [&](size_t r) { return a.wr[r] * __ldcg(a.x + r); });
    if (!grid_sync(a, B_LEVELS64, bst)) break;
    // ---- E, F: r64 = b - A x per owned skewer; r = r64, z = G G^T r
    rz = 0.0;
    rr = 0.0;
    for (int blk = blockIdx.x; blk < a.n_blocks; blk += G) {
      double acc[RPT];
      block_product<double, UF64, NB>(a, blk, a.optr, a.oidx, a.olev, a.op64, a.V64, s_off, s_p64,
                                  s_cnt, acc);
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
      block_precond<BAND>(a, a.L + (size_t)blk * a.S, ns, rs, ts, zk);
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
        a.part[(size_t)P2 + 2 * blockIdx.x] = b1;
        a.part[(size_t)P2 + 2 * blockIdx.x + 1] = b2;
      }
    }
    if (!grid_sync(a, B_UPDATE, bst)) break;
    {
      const double2 t2 = partial_total2(a.part + P2, G, tot);
      if (tid == 0) update_scalars(sS, a, t2.x, t2.y);
      __syncthreads();
    }
  }
  if (blockIdx.x == 0 && tid == 0) {
    a.pt[PT_KERNEL] += global_ns() - a.pt[PT_START];
    sS.skip_update = 1;
    *a.S_ = sS;
  }
}

// a b for float pairs, renormalised (the product's error by FMA, the cross
// terms in FP32).
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  ff r;
  fast_two_sum(p, e, r.h, r.l);
  return r;
}

// The FP64-accurate product of block blk in float pairs: out[t] = sum over
// the outer list of the skewer of record t of P V[(lev - 1) n + idx n_per +
// k] with P and V float pairs (V the levels of the update, stored as float
// pairs), the lists staged NB_R entries at a time as in block_product.
__device__ __forceinline__ void block_product_ff(const PersistArgs& a, int blk, const float2* V,
                                                size_t* s_off, float2* s_p, int* s_cnt,
                                                ff (&out)[RPT]) {
  const int m = a.g * a.n_per;
  const size_t n = (size_t)a.n;
#pragma unroll
  for (int t = 0; t < RPT; ++t) out[t] = ff{0.f, 0.f};
  int jj[RPT], kk[RPT];
#pragma unroll
  for (int t = 0; t < RPT; ++t) {
    const int i = threadIdx.x + t * NT;
    jj[t] = i < m ? i / a.n_per : -1;
    kk[t] = i < m ? i - jj[t] * a.n_per : 0;
  }
  for (int c0 = 0;; c0 += NB_R) {
    __syncthreads();
    if (threadIdx.x < MAX_G) {
      const int j = threadIdx.x;
      const int s = j < a.g ? skewer_of(a, blk, j) : -1;
      const int len = s >= 0 ? a.optr[s + 1] - a.optr[s] : 0;
      s_cnt[j] = max(0, min(NB_R, len - c0));
      s_cnt[MAX_G + j] = len - c0 > NB_R;
    }
    for (int t = threadIdx.x; t < a.g * NB_R; t += NT) {
      const int j = t / NB_R, e = t - j * NB_R;
      const int s = skewer_of(a, blk, j);
      if (s < 0) continue;
      const int q = a.optr[s] + c0 + e;
      if (q < a.optr[s + 1]) {
        s_off[t] = (size_t)(a.olev[q] - 1) * n + (size_t)a.oidx[q] * a.n_per;
        s_p[t] = a.op_ff[q];
      }
    }
    __syncthreads();
    int cnt[RPT];
#pragma unroll
    for (int t = 0; t < RPT; ++t) cnt[t] = jj[t] >= 0 ? s_cnt[jj[t]] : 0;
    int cmax = 0;
#pragma unroll
    for (int t = 0; t < RPT; ++t) cmax = max(cmax, cnt[t]);
    for (int e = 0; e < cmax; e += UF64) {
      float2 v[RPT][UF64];
#pragma unroll
      for (int t = 0; t < RPT; ++t)
#pragma unroll
        for (int u = 0; u < UF64; ++u)
          v[t][u] = e + u < cnt[t] ? __ldcg(V + s_off[jj[t] * NB_R + e + u] + kk[t])
                                   : make_float2(0.f, 0.f);
#pragma unroll
      for (int t = 0; t < RPT; ++t)
#pragma unroll
        for (int u = 0; u < UF64; ++u)
          if (e + u < cnt[t]) {
            const float2 pv = s_p[jj[t] * NB_R + e + u];
            ff_mac(out[t].h, out[t].l, ff{pv.x, pv.y}, ff{v[t][u].x, v[t][u].y});
          }
    }
    int more = 0;
    for (int j = 0; j < MAX_G; ++j) more |= s_cnt[MAX_G + j];
    if (!more) break;
  }
}

// ---- resident form: one block per CTA, the block's vectors in shared memory
//
// With at most one block per CTA (the cooperative grid holds every block),
// each CTA keeps its block's FP32 vectors p, z, q (record-local order j n_per
// + k), r (slot order), the FP64 iterate x, the FP32 coefficients and its
// skewers' FP32 neighbour lists in shared memory for the whole solve: the
// phases then read global memory only for the neighbours' levels (B), the
// factor (C) and the partials, and the levels they publish (A, D).  x goes
// back to global memory at the end.  Same recurrence, same sums in the same
// order as the general form.
constexpr int NI = 512;   // product items of a block kept in shared memory
constexpr int GI = 4;     // skewers per block of the item form at most

// Shared-memory layout of the resident form (bytes from the dynamic base).
struct ResLayout {
  static constexpr size_t xs = 0;                                   // double[MAX_S]
  static constexpr size_t us = xs + MAX_S * sizeof(double);         // double[MAX_S]
  static constexpr size_t ps = us + MAX_S * sizeof(double);         // float[MAX_S] x 8
  static constexpr size_t icoef = ps + 8 * MAX_S * sizeof(float);   // float4[NI]
  static constexpr size_t ioff = icoef + NI * sizeof(float4);       // uint32[NI]
  static constexpr size_t loc = ioff + NI * sizeof(unsigned int);   // int[MAX_S]
  static constexpr size_t nit = loc + MAX_S * sizeof(int);          // int (items)
  static constexpr size_t sk = nit + 4 * sizeof(int);               // int[MAX_G]
  static constexpr size_t lh = (sk + MAX_G * sizeof(int) + 15) / 16 * 16;  // half[(band + 1) S]
  static size_t bytes(int band, int S) { return lh + ((size_t)(band + 1) * S * 2 + 15) / 16 * 16; }
};

// z = G G^T r over the CTA's block from r in shared memory, with the block's
// factor in shared memory in FP16 (plane m, slot i at Lh[m S + i]; a
// preconditioner needs no more: M^-1 = G G^T stays symmetric positive
// definite whatever the rounding of G).
template <int BAND>
__device__ __forceinline__ void block_precond_h(const PersistArgs& a, const __half* Lh,
                                                const float* rs, float* ts, float (&zk)[RPT]) {
  const int band = BAND >= 0 ? BAND : a.band;
  const int S = a.S;
#pragma unroll
  for (int t = 0; t < RPT; ++t) {
    const int i = threadIdx.x + t * NT;
    if (i < S) {
      float v = 0.f;
#pragma unroll(BAND >= 0 ? BAND + 1 : 1)
      for (int m = 0; m <= (BAND >= 0 ? BAND : MAX_BAND); ++m)
        if (m <= band && i + m < S) v = fmaf(__half2float(Lh[m * S + i + m]), rs[i + m], v);
      ts[i] = v;
    }
  }
  __syncthreads();
#pragma unroll
  for (int t = 0; t < RPT; ++t) {
    const int i = threadIdx.x + t * NT;
    float v = 0.f;
    if (i < S) {
#pragma unroll(BAND >= 0 ? BAND + 1 : 1)
      for (int m = 0; m <= (BAND >= 0 ? BAND : MAX_BAND); ++m)
        if (m <= band && i - m >= 0) v = fmaf(__half2float(Lh[m * S + i]), ts[i - m], v);
    }
    zk[t] = v;
  }
}

template <int BAND>
__global__ void __launch_bounds__(NT, 2) k_mixed_resident(PersistArgs a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  ff* xs = reinterpret_cast<ff*>(smraw + ResLayout::xs);  // the iterate, float pairs
  double* us = reinterpret_cast<double*>(smraw + ResLayout::us);
  float4* icoef = reinterpret_cast<float4*>(smraw + ResLayout::icoef);
  unsigned int* ioff = reinterpret_cast<unsigned int*>(smraw + ResLayout::ioff);
  int* s_nit = reinterpret_cast<int*>(smraw + ResLayout::nit);
  float* ps = reinterpret_cast<float*>(smraw + ResLayout::ps);
  float* zs = ps + MAX_S;
  float* qs = zs + MAX_S;
  float* rs = qs + MAX_S;   // slot order
  float* ts = rs + MAX_S;   // scratch: u (A), t = G^T r (C, F)
  float* wls = ts + MAX_S;  // FP32 coefficients
  float* wrs = wls + MAX_S;
  float* es = wrs + MAX_S;
  int* loc = reinterpret_cast<int*>(smraw + ResLayout::loc);  // slot -> record-local index
  int* sk = reinterpret_cast<int*>(smraw + ResLayout::sk);
  __half* Lh = reinterpret_cast<__half*>(smraw + ResLayout::lh);
  __shared__ MixedState sS;
  __shared__ double red[NT / 32];
  __shared__ double tot[2];
  __shared__ ff s_alpha;  // alpha as a float pair (x update)
  __shared__ float s_ab;  // alpha or beta in FP32
  __shared__ size_t s_off[MAX_G * NB_R];  // staged FP64 lists (the update's residual)
  __shared__ double s_p64[MAX_G * NB_R];
  __shared__ int s_cnt[2 * MAX_G];
  const int tid = threadIdx.x;
  const int G = gridDim.x;
  const int P2 = (G + 1) & ~1;
  const int blk = blockIdx.x;
  const int npr = a.n_per;
  const int m = a.g * npr;  // records of the block (record-local index j n_per + k)
  const size_t n = (size_t)a.n;
  const size_t ns = (size_t)a.n_blocks * a.S;
  BarState bst;  // barrier state (thread 0)
  if (tid == 0) sS = *a.S_;
  if (tid == 0 && blockIdx.x == 0) {
    const unsigned long long now = global_ns();
    a.pt[PT_LAST] = now;
    a.pt[PT_START] = now;
    a.pt[PT_GRID] = gridDim.x;
    a.pt[PT_LAUNCHES] += 1;
  }
  if (tid < MAX_G) sk[tid] = tid < a.g ? skewer_of(a, blk, tid) : -1;
  {  // the block's product items
    const size_t i0 = (size_t)blk * NI;
    const int ni = a.it_cnt[blk];
    if (tid == 0) {
      s_nit[0] = ni;
      s_nit[1] = a.it_own[blk];
    }
    for (int e = tid; e < ni; e += NT) {
      ioff[e] = a.it_off[i0 + e];
      icoef[e] = a.it_coef[i0 + e];
    }
  }
  __syncthreads();
  for (int i = tid; i < m; i += NT) {
    const int j = i / npr;
    const int s = sk[j];
    if (s < 0) {
      xs[i] = ff{0.f, 0.f};
      ps[i] = zs[i] = qs[i] = wls[i] = wrs[i] = es[i] = 0.f;
      continue;
    }
    const size_t r = (size_t)s * npr + (i - j * npr);
    xs[i] = ff_from_double(a.x[r]);
    ps[i] = a.p[r];
    zs[i] = a.z[r];
    qs[i] = 0.f;
    wls[i] = (float)a.wl[r];
    wrs[i] = (float)a.wr[r];
    es[i] = (float)a.e[r];
  }
  {  // the block's factor, FP16
    const int nl = (a.band + 1) * a.S;
    for (int i = tid; i < nl; i += NT) {
      const int mm = i / a.S;
      Lh[i] = __float2half_rn(a.L[(size_t)mm * ns + (size_t)blk * a.S + (i - mm * a.S)]);
    }
  }
  for (int i = tid; i < a.S; i += NT) {
    const int rec = record_of(a, blk, i);
    int li = -1;
    float rv = 0.f;
    if (rec >= 0) {
      const int s = rec / npr;
      for (int j = 0; j < a.g; ++j)
        if (sk[j] == s) li = j * npr + (rec - s * npr);
      rv = a.r[rec];
    }
    loc[i] = li;
    rs[i] = rv;
  }
  __syncthreads();
  // the thread's records (A, B): i = tid + t NT, pixel k of skewer j
  int jj[RPT], kk[RPT];
  size_t rg[RPT];  // global record (valid when jj >= 0)
#pragma unroll
  for (int t = 0; t < RPT; ++t) {
    const int i = tid + t * NT;
    jj[t] = -1;
    kk[t] = 0;
    rg[t] = 0;
    if (i < m && sk[i / npr] >= 0) {
      jj[t] = i / npr;
      kk[t] = i - jj[t] * npr;
      rg[t] = (size_t)sk[jj[t]] * npr + kk[t];
    }
  }
  // The levels of u = wr z (FP32) of the block's skewers from zs (record
  // order; ts is the scratch for u).
  auto levels_z = [&]() {
    __syncthreads();
#pragma unroll
    for (int t = 0; t < RPT; ++t)
      if (jj[t] >= 0) ts[tid + t * NT] = wrs[tid + t * NT] * zs[tid + t * NT];
    __syncthreads();
#pragma unroll
    for (int t = 0; t < RPT; ++t) {
      const int i = tid + t * NT;
      if (jj[t] < 0) continue;
      const int k = kk[t];
      float acc = ts[i];
      a.V32[rg[t]] = acc;
      for (int l = 1; l <= a.ilmax; ++l) {
        float v = 0.f;
        if (k + l < npr) v = ts[i + l];
        if (k - l >= 0) v += ts[i - l];
        acc = fmaf(a.taps32[l], v, acc);
        a.V32[(size_t)l * n + rg[t]] = acc;
      }
    }
  };
  // Two grid barriers per iteration (Chronopoulos and Gear's arrangement of
  // the same recurrence): the product phase forms w = A32 z from the
  // published levels of z and moves both directions, p = z + beta p and
  // q = w + beta q (= A32 p), so p.q is known at its barrier; the step phase
  // then updates x and r, applies the preconditioner, publishes the levels of
  // the new z and the partials of r.z and |r|^2 at the next barrier.
  // The product w = A32 z: each (neighbour, level) row the block's skewers
  // use is loaded once and applied to all of them: thread (part, k) takes
  // pixel k of a share of the block's items, UFI rows in flight, one
  // accumulator per skewer (acc).  The rows of the block's own skewers (the
  // first items) are done between the arrival at the barrier that publishes
  // the levels and its wait; the others after it.
  const int tk = NT / npr;  // threads per pixel
  const int kq = tid % npr, part = tid / npr;
  float acc[GI];
  auto product_rows = [&](int e0, int e1) {
    for (int e = e0; e < e1; e += UFI) {
      float v[UFI];
#pragma unroll
      for (int u = 0; u < UFI; ++u) v[u] = e + u < e1 ? __ldcg(a.V32 + ioff[e + u] + kq) : 0.f;
#pragma unroll
      for (int u = 0; u < UFI; ++u)
        if (e + u < e1) {
          const float4 c = icoef[e + u];
          acc[0] = fmaf(c.x, v[u], acc[0]);
          acc[1] = fmaf(c.y, v[u], acc[1]);
          acc[2] = fmaf(c.z, v[u], acc[2]);
          acc[3] = fmaf(c.w, v[u], acc[3]);
        }
    }
  };
  auto own_rows = [&]() {
#pragma unroll
    for (int j = 0; j < GI; ++j) acc[j] = 0.f;
    const int no = s_nit[1];
    product_rows(part * no / tk, (part + 1) * no / tk);
  };
  levels_z();
  grid_arrive(a, B_LEVELS, bst);
  own_rows();
  if (grid_wait(a, B_LEVELS, bst)) {
    for (int k = 0; k < N_CALIB; ++k) grid_sync(a, B_CALIB, bst);
  }
  while (!sS.done && sS.iter < a.max_iter) {
      const int it = sS.iter + 1;
      // ---- product: w = A32 z, p = z + beta p, q = w + beta q, partial p.q;
      // the NT / n_per shares of a pixel are summed in order through shared
      // memory (us, free in this phase).
      ff dq{0.f, 0.f};
      {
        if (tid == 0) s_ab = (float)sS.beta;
        float* red_w = reinterpret_cast<float*>(us);  // (NT / n_per) x GI x n_per
        const int ni = s_nit[0] - s_nit[1], i0 = s_nit[1];  // the other blocks' rows
        product_rows(i0 + part * ni / tk, i0 + (part + 1) * ni / tk);
#pragma unroll
        for (int j = 0; j < GI; ++j) red_w[(part * GI + j) * npr + kq] = acc[j];
        __syncthreads();  // red_w, s_ab
        const float beta = s_ab;
#pragma unroll
        for (int t = 0; t < RPT; ++t) {
          if (jj[t] < 0) continue;
          const int i = tid + t * NT;
          float sum = 0.f;
          for (int pp = 0; pp < tk; ++pp) sum += red_w[(pp * GI + jj[t]) * npr + kk[t]];
          const float zv = zs[i];
          const float wv = fmaf(wls[i], sum, es[i] * zv);
          const float pv = fmaf(beta, ps[i], zv);
          const float qv = fmaf(beta, qs[i], wv);
          ps[i] = pv;
          qs[i] = qv;
          ff_acc_prod(dq, pv, qv);
        }
      }
      {
        const double bs = block_sum_ff(dq, red);
        if (tid == 0) a.part[blk] = bs;
      }
      if (!grid_sync(a, B_PRODUCT, bst)) break;
      // ---- step: alpha; x, r, z of the block; levels of z; partials
      const double pq = partial_total(a.part, G, tot);
      if (tid == 0) {
        const double al = sS.rz / pq;
        tot[0] = al;
        s_alpha = ff_from_double(al);
        s_ab = (float)al;
      }
      __syncthreads();
      const double alpha_d = tot[0];
      const float alpha = s_ab;
      const ff alpha_ff = s_alpha;
      ff rz{0.f, 0.f}, rr{0.f, 0.f};
      int li[RPT];
#pragma unroll
      for (int t = 0; t < RPT; ++t) {
        const int i = tid + t * NT;
        li[t] = i < a.S ? loc[i] : -1;
        if (li[t] >= 0) {
          const int l = li[t];
          rs[i] = fmaf(-alpha, qs[l], rs[i]);
          ff_mac(xs[l].h, xs[l].l, alpha_ff, ff{ps[l], 0.f});
        }
      }
      __syncthreads();
      {
        float zk[RPT];
        block_precond_h<BAND>(a, Lh, rs, ts, zk);
#pragma unroll
        for (int t = 0; t < RPT; ++t) {
          if (li[t] < 0) continue;
          const float ri = rs[tid + t * NT];
          zs[li[t]] = zk[t];
          ff_acc_prod(rz, ri, zk[t]);
          ff_acc_prod(rr, ri, ri);
        }
      }

      {
        const double b1 = block_sum_ff(rz, red);
        const double b2 = block_sum_ff(rr, red);
        if (tid == 0) {
          a.part[(size_t)P2 + 2 * blk] = b1;
          a.part[(size_t)P2 + 2 * blk + 1] = b2;
        }
      }
      levels_z();
      grid_arrive(a, B_STEP, bst);
      own_rows();
      if (!grid_wait(a, B_STEP, bst)) break;
      {
        const double2 t2 = partial_total2(a.part + P2, G, tot);
        if (tid == 0) step_scalars(sS, a, it, alpha_d, pq, t2.x, t2.y);
        __syncthreads();
      }
      if (!sS.need_update) continue;
      // ---- FP64-accurate update in float pairs (GB300 issues FP64 at 1/64 of
      // FP32): levels of u = wr x, stored as float pairs in the FP64 levels'
      // buffer
      float2* ufs = reinterpret_cast<float2*>(us);
      float2* V2 = reinterpret_cast<float2*>(a.V64);
#pragma unroll
      for (int t = 0; t < RPT; ++t)
        if (jj[t] >= 0) {
          const float2 w = a.wr_ff[rg[t]];
          const ff u = ff_mul(ff{w.x, w.y}, xs[tid + t * NT]);
          ufs[tid + t * NT] = make_float2(u.h, u.l);
        }
      __syncthreads();
#pragma unroll
      for (int t = 0; t < RPT; ++t) {
        const int i = tid + t * NT;
        if (jj[t] < 0) continue;
        const int k = kk[t];
        ff acc{ufs[i].x, ufs[i].y};
        V2[rg[t]] = make_float2(acc.h, acc.l);
        for (int l = 1; l <= a.olmax; ++l) {
          ff v{0.f, 0.f};
          if (k + l < npr) v = ff{ufs[i + l].x, ufs[i + l].y};
          if (k - l >= 0) v = ff_add(v, ff{ufs[i - l].x, ufs[i - l].y});
          const float2 tp = a.taps64_ff[l];
          ff_mac(acc.h, acc.l, ff{tp.x, tp.y}, v);
          V2[(size_t)l * n + rg[t]] = make_float2(acc.h, acc.l);
        }
      }
      if (!grid_sync(a, B_LEVELS64, bst)) break;
      // r64 = b - A x of the block (into us); r = r64, z = G G^T r, levels of z
      {
        ff acc[RPT];
        block_product_ff(a, blk, reinterpret_cast<const float2*>(a.V64), s_off,
                         reinterpret_cast<float2*>(s_p64), s_cnt, acc);
#pragma unroll
        for (int t = 0; t < RPT; ++t) {
          if (jj[t] < 0) continue;
          const int i = tid + t * NT;
          const float2 wl = a.wl_ff[rg[t]], e = a.e_ff[rg[t]], b = a.b_ff[rg[t]];
          const ff y = ff_add(ff_mul(ff{wl.x, wl.y}, acc[t]), ff_mul(ff{e.x, e.y}, xs[i]));
          const ff r = ff_sub(ff{b.x, b.y}, y);
          us[i] = (double)r.h + (double)r.l;
        }
      }
      __syncthreads();
      ff rz_u{0.f, 0.f};
      double rr_u = 0.0;
#pragma unroll
      for (int t = 0; t < RPT; ++t) {
        const int i = tid + t * NT;
        if (i >= a.S) continue;
        float rv = 0.f;
        if (li[t] >= 0) {
          const double rd = us[li[t]];
          rv = (float)rd;
          rr_u = fma(rd, rd, rr_u);
        }
        rs[i] = rv;
      }
      __syncthreads();
      {
        float zk[RPT];
        block_precond_h<BAND>(a, Lh, rs, ts, zk);
#pragma unroll
        for (int t = 0; t < RPT; ++t) {
          if (li[t] < 0) continue;
          zs[li[t]] = zk[t];
          ff_acc_prod(rz_u, rs[tid + t * NT], zk[t]);
        }
      }
      {
        const double b1 = block_sum_ff(rz_u, red);
        const double b2 = block_sum<NT>(rr_u, red);
        if (tid == 0) {
          a.part[(size_t)P2 + 2 * blk] = b1;
          a.part[(size_t)P2 + 2 * blk + 1] = b2;
        }
      }
      levels_z();
      grid_arrive(a, B_UPDATE, bst);
      own_rows();
      if (!grid_wait(a, B_UPDATE, bst)) break;
      {
        const double2 t2 = partial_total2(a.part + P2, G, tot);
        if (tid == 0) update_scalars(sS, a, t2.x, t2.y);
        __syncthreads();
      }
    }
  // the iterate back to global memory (record order)
#pragma unroll
  for (int t = 0; t < RPT; ++t)
    if (jj[t] >= 0) a.x[rg[t]] = (double)xs[tid + t * NT].h + (double)xs[tid + t * NT].l;
  if (blockIdx.x == 0 && tid == 0) {
    a.pt[PT_KERNEL] += global_ns() - a.pt[PT_START];
    sS.skip_update = 1;
    *a.S_ = sS;
  }
}

// Product items of one block per CTA (NT threads): the entries of its
// skewers' FP32 lists (at most NE_ITEMS) as (offset of the (neighbour,
// level) row, skewer j, factor), sorted by (row of another block, offset)
// (bitonic, in shared memory), equal offsets merged into one item with a
// factor per skewer: the rows of the block's own skewers come first.
// cnt[blk] = the block's items, own[blk] = those on its own skewers;
// cnt[n_blocks] = the largest count over the blocks, or NI + 1 when a block
// has too many entries or items.  Offsets are below 2^31.
constexpr int NE_ITEMS = 1024;
__global__ void __launch_bounds__(NT) k_build_items(int g, int n_per, int n,
                                                    const int* __restrict__ bsk,
                                                    const int* __restrict__ ptr,
                                                    const int* __restrict__ idx,
                                                    const int* __restrict__ lev,
                                                    const float* __restrict__ p32,
                                                    int* __restrict__ cnt,
                                                    int* __restrict__ own,
                                                    unsigned int* __restrict__ ioff,
                                                    float4* __restrict__ icoef) {
  __shared__ unsigned int key[NE_ITEMS];
  __shared__ unsigned int val[NE_ITEMS];  // j << 28 | entry index within the block
  __shared__ int base[GI + 1], sk[GI];
  __shared__ int scan[NE_ITEMS];
  __shared__ int n_own;
  const int blk = blockIdx.x, tid = threadIdx.x;
  if (tid == 0) {
    int c = 0;
    for (int j = 0; j < GI; ++j) {
      base[j] = c;
      const int s = j < g ? (bsk ? bsk[(size_t)blk * g + j] : (j == 0 ? blk : -1)) : -1;
      sk[j] = s;
      if (s >= 0) c += ptr[s + 1] - ptr[s];
    }
    base[GI] = c;
    n_own = 0;
  }
  __syncthreads();
  const int total = base[GI];
  if (total > NE_ITEMS) {
    if (tid == 0) {
      cnt[blk] = 0;
      atomicMax(cnt + gridDim.x, NI + 1);
    }
    return;
  }
  for (int i = tid; i < NE_ITEMS; i += NT) {
    unsigned int k = 0xffffffffu, v = 0;
    if (i < total) {
      int j = 0;
      while (j + 1 < GI && i >= base[j + 1]) ++j;
      const int q = ptr[sk[j]] + (i - base[j]);
      const int nb = idx[q];
      bool mine = false;
      for (int j2 = 0; j2 < GI; ++j2) mine |= nb == sk[j2];
      k = (unsigned int)((size_t)(lev[q] - 1) * n + (size_t)nb * n_per) |
          (mine ? 0u : 0x80000000u);
      v = ((unsigned int)j << 28) | (unsigned int)q;
    }
    key[i] = k;
    val[i] = v;
  }
  __syncthreads();
  // bitonic sort of (key, val) by key, ascending (keys are unique per skewer,
  // so equal keys differ in j: ties ordered by val for a fixed order)
  for (int size = 2; size <= NE_ITEMS; size <<= 1)
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = tid; i < NE_ITEMS / 2; i += NT) {
        const int lo = 2 * i - (i & (stride - 1));
        const int hi = lo + stride;
        const bool up = (lo & size) == 0;
        const unsigned int ka = key[lo], kb = key[hi], va = val[lo], vb = val[hi];
        const bool gt = ka > kb || (ka == kb && va > vb);
        if (gt == up) {
          key[lo] = kb;
          key[hi] = ka;
          val[lo] = vb;
          val[hi] = va;
        }
      }
      __syncthreads();
    }
  // item index of each entry: the count of distinct keys before it
  for (int i = tid; i < NE_ITEMS; i += NT)
    scan[i] = (i < total && (i == 0 || key[i] != key[i - 1])) ? 1 : 0;
  __syncthreads();
  for (int off = 1; off < NE_ITEMS; off <<= 1) {  // inclusive scan (Hillis-Steele)
    int v[NE_ITEMS / NT];
    for (int t = 0; t < NE_ITEMS / NT; ++t) {
      const int i = tid + t * NT;
      v[t] = scan[i] + (i >= off ? scan[i - off] : 0);
    }
    __syncthreads();
    for (int t = 0; t < NE_ITEMS / NT; ++t) scan[tid + t * NT] = v[t];
    __syncthreads();
  }
  const int n_items = total > 0 ? scan[total - 1] : 0;
  if (n_items > NI) {
    if (tid == 0) {
      cnt[blk] = 0;
      atomicMax(cnt + gridDim.x, NI + 1);
    }
    return;
  }
  const size_t o = (size_t)blk * NI;
  for (int e = tid; e < n_items; e += NT) icoef[o + e] = make_float4(0.f, 0.f, 0.f, 0.f);
  __syncthreads();
  for (int i = tid; i < total; i += NT) {
    const int it = scan[i] - 1;
    const int j = (int)(val[i] >> 28);
    const int q = (int)(val[i] & 0x0fffffffu);
    if (i == 0 || key[i] != key[i - 1]) {
      ioff[o + it] = key[i] & 0x7fffffffu;
      if (!(key[i] & 0x80000000u)) atomicAdd(&n_own, 1);
    }
    reinterpret_cast<float*>(icoef + o + it)[j] = p32[q];
  }
  __syncthreads();
  if (tid == 0) {
    cnt[blk] = n_items;
    own[blk] = n_own;
    atomicMax(cnt + gridDim.x, n_items);
  }
}

// out = in as float pairs.
__global__ void k_to_ff(size_t n, const double* __restrict__ in, float2* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const ff f = ff_from_double(in[i]);
    out[i] = make_float2(f.h, f.l);
  }
}

void to_ff(DevBuf<float2>& out, const double* in, size_t n, cudaStream_t st) {
  out.alloc(n);
  k_to_ff<<<(unsigned)std::min<size_t>(1024, (n + 255) / 256), 256, 0, st>>>(n, in, out.p);
  DS_CHECK_LAUNCH();
}

// Resident CTAs per SM of a kernel at `smem` dynamic bytes (0: does not fit).
int resident_per_sm(const void* fn, size_t smem) {
  cudaFuncAttributes fa;
  DS_CUDA(cudaFuncGetAttributes(&fa, fn));
  int dev = 0, optin = 0;
  DS_CUDA(cudaGetDevice(&dev));
  DS_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  if (fa.sharedSizeBytes + smem > (size_t)optin) return 0;
  DS_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                               (int)cudaSharedmemCarveoutMaxShared));
  if (smem > 48 * 1024)
    DS_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  DS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, NT, smem));
  return per_sm;
}

template <int BAND>
const void* kernel_of(bool resident) {
  return resident ? (const void*)k_mixed_resident<BAND> : (const void*)k_mixed_persistent<BAND>;
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
  auto pick = [&](bool resident) {
    return band == 16 ? kernel_of<16>(resident)
                      : band == 2 ? kernel_of<2>(resident) : kernel_of<-1>(resident);
  };
  // The resident form when every block gets its own resident CTA and the
  // longest FP32 neighbour list of a block fits in shared memory.
  // The resident form's product items, built on the device once per
  // preconditioner and inner cutoff (k_build_items): per block, the distinct
  // (neighbour, level) rows its skewers' FP32 lists name, ordered by offset,
  // with each skewer's factor, in slots of NI per block.
  const bool off31 = (double)(g.inner.lmax + 1) * (double)op->n < 2147483647.0;
  if (g.res_pc != pc || g.res_cut != g.inner.cut) {
    g.res_max_list = NI + 1;  // unusable unless built
    if (off31 && pc->g <= GI && NT % g.n_per == 0 && g.inner.idx.n < (1u << 28)) {
      g.it_cnt.alloc(pc->n_sk + 1);  // last: the largest count (or an overflow mark)
      g.it_own.alloc(pc->n_sk);
      g.it_off.alloc((size_t)pc->n_sk * NI);
      g.it_coef.alloc((size_t)pc->n_sk * NI);
      DS_CUDA(cudaMemsetAsync(g.it_cnt.p, 0, g.it_cnt.bytes(), st));
      k_build_items<<<pc->n_sk, NT, 0, st>>>(pc->g, g.n_per, op->n, pc->bsk.p, g.inner.ptr.p,
                                             g.inner.idx.p, g.inner.lev.p, g.inner.p32.p,
                                             g.it_cnt.p, g.it_own.p, g.it_off.p,
                                             g.it_coef.p);
      DS_CHECK_LAUNCH();
      int mx = 0;
      DS_CUDA(cudaMemcpyAsync(&mx, g.it_cnt.p + pc->n_sk, sizeof(int), cudaMemcpyDeviceToHost,
                              st));
      DS_CUDA(cudaStreamSynchronize(st));
      g.res_max_list = mx;
    }
    g.res_pc = pc;
    g.res_cut = g.inner.cut;
  }
  const size_t res_bytes = ResLayout::bytes(band, pc->n_per);
  static int per_sm0[3] = {-1, -1, -1};
  static int per_sm1[3] = {-1, -1, -1};
  static size_t res_last[3] = {0, 0, 0};
  const int bi = band == 16 ? 0 : band == 2 ? 1 : 2;
  if (per_sm0[bi] < 0) per_sm0[bi] = resident_per_sm(pick(false), 0);
  if (res_last[bi] != res_bytes) {
    per_sm1[bi] = resident_per_sm(pick(true), res_bytes);
    res_last[bi] = res_bytes;
  }
  const int nsm = op->ctx->num_sms;
  // the item form: 32-bit offsets into the levels, <= GI skewers per block,
  // n_per dividing the CTA, every block's items in shared memory
  const bool resident = g.res_max_list <= NI && per_sm1[bi] * nsm >= pc->n_sk;
  const int grid = resident ? pc->n_sk : std::min(per_sm0[bi] * nsm, pc->n_sk);
  if (grid <= 0) return false;
  g.p_part.alloc((size_t)3 * grid + 1);
  const size_t n_pt = PT_CTA + 8 * (size_t)grid;
  if (g.p_time.n < n_pt) {  // the phase timers accumulate until read
    g.p_time.alloc(n_pt);
    DS_CUDA(cudaMemsetAsync(g.p_time.p, 0, g.p_time.bytes(), st));
  }
  const size_t n_sync = BAR_WORDS;
  g.p_sync.alloc(n_sync);
  DS_CUDA(cudaMemsetAsync(g.p_sync.p, 0, n_sync * sizeof(int), st));
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
  a.bar = reinterpret_cast<unsigned int*>(g.p_sync.p);
  a.err = g.p_sync.p + 1;
  a.limit = op->ctx->wait_limit > 0 ? op->ctx->wait_limit : 4000000000LL;
  a.pt = g.p_time.p;
  a.it_cnt = g.it_cnt.p;
  a.it_own = g.it_own.p;
  a.it_off = g.it_off.p;
  a.it_coef = g.it_coef.p;
  if (!g.ff_b.p) {  // float-pair copies for the update (fixed for the grid's life)
    const size_t np = (size_t)op->pix.n_pad;
    to_ff(g.ff_wl, sv.wl, np, st);
    to_ff(g.ff_wr, sv.wr, np, st);
    to_ff(g.ff_e, sv.e, np, st);
    to_ff(g.ff_b, sv.b, np, st);
    to_ff(g.ff_op, g.outer.p64.p, g.outer.p64.n, st);
    to_ff(g.ff_taps, g.taps64.p, g.taps64.n, st);
  }
  a.wl_ff = g.ff_wl.p;
  a.wr_ff = g.ff_wr.p;
  a.e_ff = g.ff_e.p;
  a.b_ff = g.ff_b.p;
  a.op_ff = g.ff_op.p;
  a.taps64_ff = g.ff_taps.p;
  void* args[] = {&a};
  DS_CUDA(cudaLaunchCooperativeKernel(pick(resident), dim3(grid), dim3(NT), args,
                                      resident ? res_bytes : 0, st));
  DS_CHECK_LAUNCH();
  return true;
}

int persistent_error(ds_operator* op, cudaStream_t st) {
  SkewerGrid& g = *op->sgrid;
  if (!g.p_sync.p) return 0;
  int code = 0;
  DS_CUDA(cudaMemcpyAsync(&code, g.p_sync.p + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
  DS_CUDA(cudaStreamSynchronize(st));
  if (code) DS_CUDA(cudaMemsetAsync(g.p_sync.p, 0, g.p_sync.bytes(), st));
  return code;
}

// The phase timers as per-visit averages (see ds_operator_get_persistent_profile).
int persistent_profile(ds_operator* op, double* out, int n, bool reset) {
  if (!op->sgrid || !op->sgrid->p_time.p) return 0;
  SkewerGrid& g = *op->sgrid;
  cudaStream_t st = op->ctx->stream;
  std::vector<unsigned long long> v(g.p_time.n);
  DS_CUDA(cudaMemcpyAsync(v.data(), g.p_time.p, v.size() * sizeof(unsigned long long),
                          cudaMemcpyDeviceToHost, st));
  DS_CUDA(cudaStreamSynchronize(st));
  if (reset) DS_CUDA(cudaMemsetAsync(g.p_time.p, 0, g.p_time.bytes(), st));
  std::vector<double> r(4 + 4 * 5 + 2, 0.0);
  const int grid = (int)v[PT_GRID];
  // the resident form's product: neighbour values loaded per product
  // (items x n_per); 0 for the general form
  if (g.it_cnt.p && g.res_max_list <= NI && g.res_pc == op->pc.get()) {
    std::vector<int> cnt(g.it_cnt.n);
    DS_CUDA(cudaMemcpyAsync(cnt.data(), g.it_cnt.p, cnt.size() * sizeof(int),
                            cudaMemcpyDeviceToHost, st));
    DS_CUDA(cudaStreamSynchronize(st));
    long long items = 0;
    for (size_t b = 0; b + 1 < cnt.size(); ++b) items += cnt[b];
    r[24] = (double)items * g.n_per;
    r[25] = (double)items;
  }
  r[0] = (double)v[PT_LAUNCHES];
  r[1] = v[PT_KERNEL] * 1e-6;  // ms
  r[2] = grid;
  if (v[PT_VISITS + B_CALIB]) r[3] = v[PT_PHASE + B_CALIB] * 1e-3 / v[PT_VISITS + B_CALIB];
  for (int c = 1; c <= 5; ++c) {
    const double vis = (double)v[PT_VISITS + c];
    double* o = r.data() + 4 + 4 * (c - 1);
    o[3] = vis;
    if (!vis) continue;
    o[0] = v[PT_PHASE + c] * 1e-3 / vis;  // us per visit (CTA 0, exit to exit)
    double sum = 0.0, mx = 0.0;
    for (int b = 0; b < grid && PT_CTA + 8 * (size_t)b + c < v.size(); ++b) {
      const double w = (double)v[PT_CTA + 8 * (size_t)b + c];
      sum += w;
      mx = std::max(mx, w);
    }
    o[1] = grid ? sum * 1e-3 / vis / grid : 0.0;  // mean CTA work, us
    o[2] = mx * 1e-3 / vis;                       // slowest CTA's work, us
  }
  const int m = std::min<int>(n, (int)r.size());
  for (int i = 0; i < m; ++i) out[i] = r[i];
  return m;
}

}  // namespace ds
