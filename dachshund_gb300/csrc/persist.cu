// Persistent form of the structured mixed-precision iteration (no reference
// counterpart; the recurrence is lib/pcg.h:27-160 with FP32 inner products
// and FP64-accurate reliable updates, as in mixed.cu).
//
// The per-kernel iteration (mixed.cu) spends most of its time waiting: each
// of its kernels moves ~20 MB in ~20 us, the launch ramp, the chains of
// dependent loads and the single CTA that reduces the partials at the end
// of each kernel dominate.  Here one cooperative launch runs every
// iteration: the CTAs stay resident and pass through phases separated by
// grid-wide barriers, each CTA keeping its own copy of the CG scalars and
// computing them from the same partials in the same order (so all copies
// agree bit for bit and no CTA has to broadcast them):
//   P1  p = z + beta p and the z-convolution levels of u = w p   (per skewer)
//   P2  q = A32 p and the partial p.q                           (per skewer)
//   P3  alpha = r.z / p.q; x += alpha p, r -= alpha q, z = G G^T r and the
//       partials r.z, |r|^2                                     (per 256 slots)
//   P4  the scalar recurrence: beta, |r|, the update test        (every CTA)
// and, when an FP64 update is due, the structured FP64 residual (P5 levels,
// P6 r64 = b - A x), the update (P7: r = r64, z = G G^T r, partials) and
// its scalars (P8).  Three barriers per iteration, three more per update.
// Data written by other CTAs during the kernel is read through L2
// (ld.global.cg), never from a possibly stale L1 line.
//
// Every barrier wait is bounded (`limit` SM clock cycles): a CTA that runs
// out records an error code, and every CTA leaves at its next barrier; the
// host reports DS_ERR_TIMEOUT.  The launch is cooperative, so all CTAs are
// resident and a barrier always completes unless a CTA has left.
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

constexpr int PT = 256;            // threads per CTA (also the slots per P3 tile)
constexpr int PT_MAX_NPER = 1024;  // pixels per skewer at most
constexpr int P_NB = 256;          // neighbour entries staged per round
constexpr int P_MAXB = 32;         // band of the cluster factor at most
constexpr int P_U = 8;             // neighbours per step in the apply phases

struct PersistArgs {
  int n, n_sk, n_per, n_slots, band, max_iter;
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
  // record-order coefficients
  const double *wl, *wr, *e, *b;
  // record-order vectors
  double* x;
  float *p, *q, *z, *r0, *r1;
  double* r64;
  // cluster factor
  const int* crec;
  const float* L;
  // state and scratch
  MixedState* S;
  double *hist, *htrue, *part;
  unsigned int *bar_count, *bar_gen;
  int* err;
  long long limit;
};

// Barrier codes: the phase whose closing barrier gave up.
enum { B_LEVELS = 1, B_PRODUCT, B_STEP, B_LEVELS64, B_RESIDUAL, B_UPDATE };

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
        __nanosleep(64);
      }
    }
    __threadfence();
    ok_s = ok && *err == 0;
  }
  __syncthreads();
  return ok_s != 0;
}

// Sum over the CTA of one value per thread, valid in every thread.
__device__ __forceinline__ double cta_total(double v, double* red, double* out) {
  const double s = block_sum<PT>(v, red);
  if (threadIdx.x == 0) *out = s;
  __syncthreads();
  const double t = *out;
  __syncthreads();
  return t;
}

// Sum of n partials (stride, offset) in a fixed order, in every CTA alike.
__device__ __forceinline__ double partial_total(const double* part, int n, int stride, int off,
                                                double* red, double* out) {
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += PT) v += __ldcg(part + (size_t)i * stride + off);
  return cta_total(v, red, out);
}

// Stages the offsets and factors of entries c0 .. c0 + cnt of a CSR row.
template <typename T>
__device__ __forceinline__ void stage_row(int c0, int cnt, const int* __restrict__ idx,
                                          const int* __restrict__ lev,
                                          const T* __restrict__ pv, size_t plane, int stride,
                                          size_t* s_off, T* s_p) {
  __syncthreads();
  for (int t = threadIdx.x; t < cnt; t += PT) {
    s_off[t] = (size_t)(lev[c0 + t] - 1) * plane + (size_t)idx[c0 + t] * stride;
    s_p[t] = pv[c0 + t];
  }
  __syncthreads();
}

// sum over the staged entries of p V[off + k] (V read through L2).
template <typename T>
__device__ __forceinline__ T staged_sum(int cnt, const size_t* s_off, const T* s_p,
                                        const T* V, int k) {
  T acc[P_U];
#pragma unroll
  for (int u = 0; u < P_U; ++u) acc[u] = T(0);
  int i = 0;
  for (; i + P_U <= cnt; i += P_U) {
    T v[P_U];
#pragma unroll
    for (int u = 0; u < P_U; ++u) v[u] = __ldcg(V + s_off[i + u] + k);
#pragma unroll
    for (int u = 0; u < P_U; ++u) acc[u] = fma(s_p[i + u], v[u], acc[u]);
  }
  for (; i < cnt; ++i) acc[0] = fma(s_p[i], __ldcg(V + s_off[i] + k), acc[0]);
  T s = T(0);
#pragma unroll
  for (int u = 0; u < P_U; ++u) s += acc[u];
  return s;
}

// z = G G^T r over one tile of PT slots (halo `band` each side) from r
// values produced by `rval` for any slot; returns the thread's own slot's
// (index, r, z) through the references.
template <class RVal>
__device__ __forceinline__ void band_tile(const PersistArgs& a, int s0, float* rs, float* ts,
                                          RVal&& rval, int& own, float& ri, float& zk) {
  const int band = a.band;
  const size_t ns = (size_t)a.n_slots;
  auto index_of = [&](int slot) -> int {
    if (slot < 0 || slot >= a.n_slots) return -1;
    return a.crec ? a.crec[slot] : slot;
  };
  __syncthreads();
  for (int i = threadIdx.x; i < PT + 2 * band; i += PT) {
    const int pos = index_of(s0 - band + i);
    rs[i] = pos >= 0 ? rval(pos) : 0.f;
  }
  __syncthreads();
  const int k = s0 + threadIdx.x;
  own = index_of(k);
  ri = rs[threadIdx.x + band];
  for (int i = threadIdx.x; i < PT + band; i += PT) {
    const int j = s0 - band + i;
    float t = 0.f;
    if (j >= 0)
      for (int m = 0; m <= band; ++m)
        if (j + m < a.n_slots) t = fmaf(a.L[(size_t)m * ns + j + m], rs[i + m], t);
    ts[i] = t;
  }
  __syncthreads();
  zk = 0.f;
  if (k < a.n_slots)
    for (int m = 0; m <= band; ++m) zk = fmaf(a.L[(size_t)m * ns + k], ts[threadIdx.x + band - m], zk);
}

__global__ void __launch_bounds__(PT) k_mixed_persistent(PersistArgs a) {
  __shared__ MixedState sS;
  __shared__ double red[PT / 32];
  __shared__ double tot;
  __shared__ __align__(16) double su64[PT_MAX_NPER];  // u of one skewer (FP64 or FP32)
  float* su = reinterpret_cast<float*>(su64);
  __shared__ size_t s_off[P_NB];
  __shared__ double s_p64[P_NB];
  __shared__ float s_p32[P_NB];
  __shared__ float rs[PT + 2 * P_MAXB];
  __shared__ float ts[PT + P_MAXB];
  const int tid = threadIdx.x;
  const size_t n = (size_t)a.n;
  const int n_tiles = (a.n_slots + PT - 1) / PT;
  if (tid == 0) sS = *a.S;
  __syncthreads();
  while (!sS.done && sS.iter <= a.max_iter + 1) {
    const int it = sS.iter + 1;
    float* rin = (it & 1) ? a.r0 : a.r1;   // rbuf[(it - 1) & 1]
    float* rout = (it & 1) ? a.r1 : a.r0;  // rbuf[it & 1]
    // ---- P1: p = z + beta p, levels of u = w p
    const float beta = (float)sS.beta;
    for (int s = blockIdx.x; s < a.n_sk; s += gridDim.x) {
      __syncthreads();
      for (int k = tid; k < a.n_per; k += PT) {
        const size_t r = (size_t)s * a.n_per + k;
        const float pv = fmaf(beta, __ldcg(a.p + r), __ldcg(a.z + r));
        a.p[r] = pv;
        su[k] = (float)a.wr[r] * pv;
      }
      __syncthreads();
      for (int k = tid; k < a.n_per; k += PT) {
        const size_t r = (size_t)s * a.n_per + k;
        float acc = su[k];
        a.V32[r] = acc;
        for (int l = 1; l <= a.ilmax; ++l) {
          float v = 0.f;
          if (k + l < a.n_per) v = su[k + l];
          if (k - l >= 0) v += su[k - l];
          acc = fmaf(a.taps32[l], v, acc);
          a.V32[(size_t)l * n + r] = acc;
        }
      }
    }
    if (!grid_sync(a, B_LEVELS)) break;
    // ---- P2: q = A32 p, partial p.q
    double dq = 0.0;
    for (int s = blockIdx.x; s < a.n_sk; s += gridDim.x) {
      const int q0 = a.iptr[s], q1 = a.iptr[s + 1];
      float acc[PT_MAX_NPER / PT];
#pragma unroll
      for (int t = 0; t < PT_MAX_NPER / PT; ++t) acc[t] = 0.f;
      for (int c0 = q0; c0 < q1; c0 += P_NB) {
        const int cnt = min(P_NB, q1 - c0);
        stage_row<float>(c0, cnt, a.iidx, a.ilev, a.ip32, n, a.n_per, s_off, s_p32);
#pragma unroll
        for (int t = 0; t < PT_MAX_NPER / PT; ++t) {
          const int k = tid + t * PT;
          if (k < a.n_per) acc[t] += staged_sum<float>(cnt, s_off, s_p32, a.V32, k);
        }
      }
#pragma unroll
      for (int t = 0; t < PT_MAX_NPER / PT; ++t) {
        const int k = tid + t * PT;
        if (k >= a.n_per) break;
        const size_t r = (size_t)s * a.n_per + k;
        const float pv = __ldcg(a.p + r);
        const float qv = fmaf((float)a.wl[r], acc[t], (float)a.e[r] * pv);
        a.q[r] = qv;
        dq = fma((double)pv, (double)qv, dq);
      }
    }
    {
      const double bs = block_sum<PT>(dq, red);
      if (tid == 0) a.part[blockIdx.x] = bs;
    }
    if (!grid_sync(a, B_PRODUCT)) break;
    // ---- P3: alpha; x, r, z over slot tiles; partials r.z, |r|^2
    const double pq = partial_total(a.part, gridDim.x, 1, 0, red, &tot);
    const double alpha_d = sS.rz / pq;
    const float alpha = (float)alpha_d;
    double rz = 0.0, rr = 0.0;
    for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) {
      int own;
      float ri, zk;
      band_tile(a, t * PT, rs, ts,
                [&](int pos) { return fmaf(-alpha, __ldcg(a.q + pos), __ldcg(rin + pos)); }, own,
                ri, zk);
      if (own >= 0) {
        rout[own] = ri;
        a.x[own] = fma(alpha_d, (double)__ldcg(a.p + own), __ldcg(a.x + own));
        a.z[own] = zk;
        rz = fma((double)ri, (double)zk, rz);
        rr = fma((double)ri, (double)ri, rr);
      }
    }
    {
      const double b1 = block_sum<PT>(rz, red);
      const double b2 = block_sum<PT>(rr, red);
      if (tid == 0) {
        a.part[(size_t)gridDim.x + 2 * blockIdx.x] = b1;
        a.part[(size_t)gridDim.x + 2 * blockIdx.x + 1] = b2;
      }
    }
    if (!grid_sync(a, B_STEP)) break;
    // ---- P4: the scalars (every CTA alike)
    {
      const double trz = partial_total(a.part + gridDim.x, gridDim.x, 2, 0, red, &tot);
      const double trr = partial_total(a.part + gridDim.x, gridDim.x, 2, 1, red, &tot);
      if (tid == 0) {
        sS.alpha = alpha_d;
        sS.pq = pq;
        sS.rz_old = sS.rz;
        sS.rz = trz;
        sS.rnorm = sqrt(trr);
        sS.iter = it;
        if (blockIdx.x == 0) a.hist[it] = sS.rnorm;
        sS.rmax = fmax(sS.rmax, sS.rnorm);
        const bool upd = update_due(&sS, it);
        sS.need_update = upd ? 1 : 0;
        sS.beta = sS.rz / sS.rz_old;
      }
      __syncthreads();
    }
    if (!sS.need_update) continue;
    // ---- P5: levels of u = w x (FP64)
    for (int s = blockIdx.x; s < a.n_sk; s += gridDim.x) {
      __syncthreads();
      for (int k = tid; k < a.n_per; k += PT) {
        const size_t r = (size_t)s * a.n_per + k;
        su64[k] = a.wr[r] * __ldcg(a.x + r);
      }
      __syncthreads();
      for (int k = tid; k < a.n_per; k += PT) {
        const size_t r = (size_t)s * a.n_per + k;
        double acc = su64[k];
        a.V64[r] = acc;
        for (int l = 1; l <= a.olmax; ++l) {
          double v = 0.0;
          if (k + l < a.n_per) v = su64[k + l];
          if (k - l >= 0) v += su64[k - l];
          acc = fma(a.taps64[l], v, acc);
          a.V64[(size_t)l * n + r] = acc;
        }
      }
    }
    if (!grid_sync(a, B_LEVELS64)) break;
    // ---- P6: r64 = b - A x (FP64)
    for (int s = blockIdx.x; s < a.n_sk; s += gridDim.x) {
      const int q0 = a.optr[s], q1 = a.optr[s + 1];
      double acc[PT_MAX_NPER / PT];
#pragma unroll
      for (int t = 0; t < PT_MAX_NPER / PT; ++t) acc[t] = 0.0;
      for (int c0 = q0; c0 < q1; c0 += P_NB) {
        const int cnt = min(P_NB, q1 - c0);
        stage_row<double>(c0, cnt, a.oidx, a.olev, a.op64, n, a.n_per, s_off, s_p64);
#pragma unroll
        for (int t = 0; t < PT_MAX_NPER / PT; ++t) {
          const int k = tid + t * PT;
          if (k < a.n_per) acc[t] += staged_sum<double>(cnt, s_off, s_p64, a.V64, k);
        }
      }
#pragma unroll
      for (int t = 0; t < PT_MAX_NPER / PT; ++t) {
        const int k = tid + t * PT;
        if (k >= a.n_per) break;
        const size_t r = (size_t)s * a.n_per + k;
        const double y = fma(a.wl[r], acc[t], a.e[r] * __ldcg(a.x + r));
        a.r64[r] = a.b[r] - y;
      }
    }
    if (!grid_sync(a, B_RESIDUAL)) break;
    // ---- P7: r = r64, z = G G^T r, partials
    rz = 0.0;
    rr = 0.0;
    for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) {
      int own;
      float ri, zk;
      band_tile(a, t * PT, rs, ts, [&](int pos) { return (float)__ldcg(a.r64 + pos); }, own,
                ri, zk);
      if (own >= 0) {
        const double rd = __ldcg(a.r64 + own);
        rout[own] = ri;
        a.z[own] = zk;
        rz = fma((double)ri, (double)zk, rz);
        rr = fma(rd, rd, rr);
      }
    }
    {
      const double b1 = block_sum<PT>(rz, red);
      const double b2 = block_sum<PT>(rr, red);
      if (tid == 0) {
        a.part[(size_t)gridDim.x + 2 * blockIdx.x] = b1;
        a.part[(size_t)gridDim.x + 2 * blockIdx.x + 1] = b2;
      }
    }
    if (!grid_sync(a, B_UPDATE)) break;
    // ---- P8: the update's scalars
    {
      const double trz = partial_total(a.part + gridDim.x, gridDim.x, 2, 0, red, &tot);
      const double trr = partial_total(a.part + gridDim.x, gridDim.x, 2, 1, red, &tot);
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
    // the next phase P3 reuses part[gridDim.x ..]: every CTA has read it
    // above, and two barriers (P1 | P2, P2 | P3) come before it is rewritten
  }
  if (blockIdx.x == 0 && tid == 0) {
    sS.skip_update = 1;
    *a.S = sS;
  }
}

}  // namespace

// The structured mixed solve's iterations as one cooperative launch; false
// when its conditions do not hold (then the caller runs the per-kernel
// iteration).  X, vectors and coefficients in record order; S initialised
// by the start kernels.
bool run_mixed_persistent(ds_operator* op, OpF32& f, const SkewerPC* pc, const SkewerVecs& sv,
                          double* X, float* r0, float* r1, int max_iter, cudaStream_t st) {
  SkewerGrid& g = *op->sgrid;
  if (!pc || pc->band > P_MAXB || g.n_per > PT_MAX_NPER || pc->n_per * pc->n_sk <= 0) return false;
  if (!g.inner.ptr.p || !g.V32.p || !g.V64.p) return false;
  int per_sm = 0;
  DS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mixed_persistent, PT, 0));
  if (per_sm <= 0) return false;
  const int grid = std::min(per_sm * op->ctx->num_sms,
                            std::max(g.n_sk, (pc->n_sk * pc->n_per + PT - 1) / PT));
  g.p_part.alloc((size_t)3 * grid);
  g.p_sync.alloc(3);
  DS_CUDA(cudaMemsetAsync(g.p_sync.p, 0, 3 * sizeof(unsigned int), st));
  PersistArgs a{};
  a.n = op->n;
  a.n_sk = g.n_sk;
  a.n_per = g.n_per;
  a.n_slots = pc->n_sk * pc->n_per;
  a.band = pc->band;
  a.max_iter = max_iter;
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
  a.z = f.z.p;
  a.r0 = r0;
  a.r1 = r1;
  a.r64 = op->r.p;
  a.crec = pc->crec.p;
  a.L = pc->L.p;
  a.S = f.state.p;
  a.hist = f.hist.p;
  a.htrue = f.htrue.p;
  a.part = g.p_part.p;
  a.bar_count = reinterpret_cast<unsigned int*>(g.p_sync.p);
  a.bar_gen = reinterpret_cast<unsigned int*>(g.p_sync.p) + 1;
  a.err = g.p_sync.p + 2;
  a.limit = op->ctx->wait_limit > 0 ? op->ctx->wait_limit : 4000000000LL;
  void* args[] = {&a};
  DS_CUDA(cudaLaunchCooperativeKernel((void*)k_mixed_persistent, dim3(grid), dim3(PT), args, 0,
                                      st));
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
