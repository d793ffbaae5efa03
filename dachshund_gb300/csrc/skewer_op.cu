// Structured FP64 form of the exact-kernel operator for skewers on a shared
// z grid (no reference counterpart; the operator is the one of
// lib/wf_vector.cc:196-251 and lib/signal_covar.h:79-86, evaluated in a
// different order).
//
// The exact kernel factorises:
//   S_ij = var_s exp(-c_perp |dxy|^2 - c_para dz^2)
//        = [var_s exp(-c_perp |dxy_ab|^2)] [exp(-c_para (z_k - z_l)^2)],
// for pixel k of skewer a and pixel l of skewer b.  When every skewer samples
// the same uniform z grid, the second factor depends on k - l only: between
// two skewers S is P_ab times a Toeplitz matrix with taps
// T_m = exp(-c_para (z_m - z_0)^2).  With the operator's cutoff (an entry is
// zero once its whole argument reaches `cut`), skewer pair (a, b) keeps the
// taps |m| <= L_ab.  So, with u = wr v,
//   (S u)_{a,k} = sum_{b near a} P_ab V_b^(L_ab)[k],
//   V_b^(L)[k] = sum_{|m| <= L} T_m u_{b,k+m}    (levels L = 0 .. lmax),
// i.e. per product one short convolution per skewer and level (lmax ~ 8 at
// the default cutoff of 40) and one FMA per (skewer pair, pixel): on the
// 262,144-pixel workload 6.4e7 FP64 FMAs against 1.9e9 exponentials of the
// pair kernels.  Every term is the FP64 product of the two factors (each
// within an ulp or two of exp), so results agree with the pair kernels to
// rounding (the sum order differs).
//
// Layout: V is (lmax + 1) x n in record order (record s n_per + k), one CTA
// per skewer and one thread per pixel in both kernels; the vectors of the
// solver stay in the operator's sorted order and are addressed through the
// record -> sorted map (op->inv).
#include <algorithm>
#include <cmath>
#include <memory>
#include <vector>

#include "ds_device.cuh"
#include "ds_ff.cuh"
#include "ds_ops.h"
#include "ds_skewer.h"

namespace ds {

void SkewerGridDeleter::operator()(SkewerGrid* p) const { delete p; }
void MapColumnsDeleter::operator()(MapColumns* p) const { delete p; }

namespace {

constexpr int NB_CHUNK = 256;  // neighbour entries staged per round

// out[t] = sum_q p[q] V[(lev[q] + lev_base) plane + idx[q] stride + k0 + t
// kstep] (t < PPT, entries with k >= kmax left 0) over the CSR row q0 .. q1:
// the row's offsets and factors are staged in shared memory a chunk at a
// time (so no V address waits on a load), and each step issues U x PPT
// independent loads (U neighbours, PPT outputs each, U chains).  Every
// thread of the CTA calls it (it synchronises).
template <typename T, int PPT, int U>
__device__ __forceinline__ void nbr_sum(int q0, int q1, const int* __restrict__ idx,
                                        const int* __restrict__ lev,
                                        const T* __restrict__ pv, int lev_base, size_t plane,
                                        int stride, const T* __restrict__ V, int k0, int kstep,
                                        int kmax, T (&out)[PPT], size_t* s_off, T* s_p) {
  T acc[PPT][U];
#pragma unroll
  for (int t = 0; t < PPT; ++t)
#pragma unroll
    for (int u = 0; u < U; ++u) acc[t][u] = T(0);
  for (int c0 = q0; c0 < q1; c0 += NB_CHUNK) {
    const int cnt = min(NB_CHUNK, q1 - c0);
    __syncthreads();
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
      s_off[t] = (size_t)(lev[c0 + t] + lev_base) * plane + (size_t)idx[c0 + t] * stride;
      s_p[t] = pv[c0 + t];
    }
    __syncthreads();
    int i = 0;
    for (; i + U <= cnt; i += U) {
      T v[U][PPT];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const size_t o = s_off[i + u];
#pragma unroll
        for (int t = 0; t < PPT; ++t) {
          const int k = k0 + t * kstep;
          v[u][t] = k < kmax ? V[o + k] : T(0);
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const T f = s_p[i + u];
#pragma unroll
        for (int t = 0; t < PPT; ++t) acc[t][u] = fma(f, v[u][t], acc[t][u]);
      }
    }
    for (; i < cnt; ++i) {
      const size_t o = s_off[i];
      const T f = s_p[i];
#pragma unroll
      for (int t = 0; t < PPT; ++t) {
        const int k = k0 + t * kstep;
        if (k < kmax) acc[t][0] = fma(f, V[o + k], acc[t][0]);
      }
    }
  }
#pragma unroll
  for (int t = 0; t < PPT; ++t) {
    T s = T(0);
#pragma unroll
    for (int u = 0; u < U; ++u) s += acc[t][u];
    out[t] = s;
  }
}

// V^(L) for L = 0..lmax of one skewer per CTA (n_per threads).
__global__ void k_sg_levels(int n_per, int lmax, size_t n, const int* __restrict__ pos,
                            const double* __restrict__ wr, const double* __restrict__ v,
                            const double* __restrict__ taps, double* __restrict__ V,
                            const int* skip) {
  if (skip && *skip) return;
  extern __shared__ double su[];
  const int k = threadIdx.x;
  const size_t r = (size_t)blockIdx.x * n_per + k;
  const size_t p = pos ? (size_t)pos[r] : r;
  const double u = wr[p] * v[p];
  su[k] = u;
  __syncthreads();
  double acc = u;
  V[r] = acc;
  for (int L = 1; L <= lmax; ++L) {
    double s = 0.0;
    if (k + L < n_per) s = su[k + L];
    if (k - L >= 0) s += su[k - L];
    acc = fma(taps[L], s, acc);
    V[(size_t)L * n + r] = acc;
  }
}

// out = A v (product) or b - A v (residual) for one skewer per CTA.
// outputs per thread (SG_PPT: FP64 residual and FP32 inner product, which
// need every thread they can get to keep loads in flight; MC_PPT: the map,
// with 3.3M outputs) and neighbours per step in the apply kernels
constexpr int SG_PPT = 1, SG_U = 8, SG32_U = 16, MC_PPT = 4, MC_U = 4;

// out = A v (product) or b - A v (residual) for one skewer per CTA
// (ceil(n_per / SG_PPT) threads, pixels k, k + blockDim, ...).
template <bool RESID>
__global__ void k_sg_apply(int n_per, size_t n, const int* __restrict__ nb_ptr,
                           const int* __restrict__ nb_idx, const int* __restrict__ nb_lev,
                           const double* __restrict__ nb_p, const double* __restrict__ V,
                           const int* __restrict__ pos, const double* __restrict__ wl,
                           const double* __restrict__ e, const double* __restrict__ v,
                           const double* __restrict__ bvec, double* __restrict__ out,
                           const int* skip, unsigned long long* prof_terms) {
  if (skip && *skip) return;
  __shared__ size_t s_off[NB_CHUNK];
  __shared__ double s_p[NB_CHUNK];
  const int a = blockIdx.x;
  const int q0 = nb_ptr[a], q1 = nb_ptr[a + 1];
  double acc[SG_PPT];
  nbr_sum<double, SG_PPT, SG_U>(q0, q1, nb_idx, nb_lev, nb_p, -1, n, n_per, V, threadIdx.x,
                                blockDim.x, n_per, acc, s_off, s_p);
#pragma unroll
  for (int t = 0; t < SG_PPT; ++t) {
    const int k = threadIdx.x + t * blockDim.x;
    if (k >= n_per) break;
    const size_t r = (size_t)a * n_per + k;
    const size_t p = pos ? (size_t)pos[r] : r;
    const double y = fma(wl[p], acc[t], e[p] * v[p]);
    out[p] = RESID ? bvec[p] - y : y;
  }
  if (prof_terms && threadIdx.x == 0)
    atomicAdd(prof_terms, (unsigned long long)(q1 - q0) * n_per);
}

// FP32 levels of the inner operator: u = wr p (FP32 vectors, sorted order).
// With beta non-null it first moves p along the CG direction, p = z + beta p
// (the step that would otherwise be a kernel of its own after the update).
__global__ void k_sg32_levels(int n_per, int lmax, size_t n, const int* __restrict__ pos,
                              const double* __restrict__ wr, float* __restrict__ p,
                              const double* beta, const float* __restrict__ z,
                              const float* __restrict__ taps, float* __restrict__ V,
                              const int* skip) {
  if (skip && *skip) return;
  extern __shared__ float sf[];
  const int k = threadIdx.x;
  const size_t r = (size_t)blockIdx.x * n_per + k;
  const size_t ps = pos ? (size_t)pos[r] : r;
  float pv = p[ps];
  if (beta) {
    pv = fmaf((float)*beta, pv, z[ps]);
    p[ps] = pv;
  }
  const float u = (float)wr[ps] * pv;
  sf[k] = u;
  __syncthreads();
  float acc = u;
  V[r] = acc;
  for (int L = 1; L <= lmax; ++L) {
    float s = 0.f;
    if (k + L < n_per) s = sf[k + L];
    if (k - L >= 0) s += sf[k - L];
    acc = fmaf(taps[L], s, acc);
    V[(size_t)L * n + r] = acc;
  }
}

// Sum over the CTA (any blockDim <= 1024) in a fixed order; valid in thread 0.
__device__ __forceinline__ double sg_cta_sum(double v, double* sm) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sm[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int k = 0; k < (int)(blockDim.x + 31) / 32; ++k) s += sm[k];
  return s;
}

// q = A32 p for one skewer per CTA, with the fused p.q of the CG step: one
// partial per skewer, summed in skewer order by the last CTA, which also
// forms alpha = num / p.q.
__global__ void k_sg32_apply(int n_per, size_t n, const int* __restrict__ nb_ptr,
                             const int* __restrict__ nb_idx, const int* __restrict__ nb_lev,
                             const float* __restrict__ nb_p, const float* __restrict__ V,
                             const int* __restrict__ pos, const double* __restrict__ wl,
                             const double* __restrict__ e, const float* __restrict__ p,
                             float* __restrict__ q, double* __restrict__ part,
                             unsigned int* counter, const double* num, double* alpha_out,
                             double* den_out, const int* skip,
                             unsigned long long* prof_terms) {
  if (skip && *skip) return;
  __shared__ double sm[32];
  __shared__ size_t s_off[NB_CHUNK];
  __shared__ float s_p[NB_CHUNK];
  const int a = blockIdx.x;
  const int q0 = nb_ptr[a], q1 = nb_ptr[a + 1];
  float acc[SG_PPT];
  nbr_sum<float, SG_PPT, SG32_U>(q0, q1, nb_idx, nb_lev, nb_p, -1, n, n_per, V, threadIdx.x,
                                 blockDim.x, n_per, acc, s_off, s_p);
  double dsum = 0.0;
#pragma unroll
  for (int t = 0; t < SG_PPT; ++t) {
    const int k = threadIdx.x + t * blockDim.x;
    if (k >= n_per) break;
    const size_t r = (size_t)a * n_per + k;
    const size_t ps = pos ? (size_t)pos[r] : r;
    const float pv = p[ps];
    const float qv = fmaf((float)wl[ps], acc[t], (float)e[ps] * pv);
    q[ps] = qv;
    dsum = fma((double)pv, (double)qv, dsum);
  }
  if (prof_terms && threadIdx.x == 0)
    atomicAdd(prof_terms, (unsigned long long)(q1 - q0) * n_per);
  if (!part) return;
  const double s = sg_cta_sum(dsum, sm);
  if (threadIdx.x == 0) part[a] = s;
  if (!last_block_arrive(counter)) return;
  double t = 0.0;
  for (int c = threadIdx.x; c < (int)gridDim.x; c += blockDim.x) t += __ldcg(part + c);
  const double pq = sg_cta_sum(t, sm);
  if (threadIdx.x == 0) {
    *den_out = pq;
    *alpha_out = *num / pq;
    *counter = 0;
  }
}

// ---- structured map --------------------------------------------------------------
constexpr int MC_QMAX = 32;  // distance classes at most

// Column (x, y) and the Z_j of a map declared a column grid, from its points
// as given (x, y, z of point c nz + j at 3 (c nz + j)).
__global__ void k_mc_info(int n, int nz, const double* __restrict__ pts,
                          double* __restrict__ cx, double* __restrict__ cy,
                          double* __restrict__ zj) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int c = p / nz, j = p % nz;
  const double* q = pts + (size_t)p * 3;
  if (j == 0) {
    cx[c] = q[0];
    cy[c] = q[1];
  }
  if (c == 0) zj[j] = q[2];
}

// Flags a point that is not at its column's (x, y) and its Z_j.
__global__ void k_mc_check(int n, int nz, const double* __restrict__ pts,
                           const double* __restrict__ cx, const double* __restrict__ cy,
                           const double* __restrict__ zj, int* __restrict__ bad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int c = p / nz, j = p % nz;
  const double* q = pts + (size_t)p * 3;
  if (q[0] != cx[c] || q[1] != cy[c] || q[2] != zj[j]) atomicOr(bad, 1);
}

// R_b^(q)[j] = sum of T_class x_{b,k} over the window pixels of Z_j whose
// distance class is < q + 1 (one thread per (skewer, Z_j)); x in caller
// order (record b n_per + k).
__global__ void k_mc_levels(int n_sk, int n_per, int nz, int W, int Q,
                            const int* __restrict__ kstart, const signed char* __restrict__ cls,
                            const double* __restrict__ taps, const double* __restrict__ x,
                            double* __restrict__ R) {
  const int j = blockIdx.y * blockDim.x + threadIdx.x;
  if (j >= nz) return;
  const int b = blockIdx.x;
  double acc[MC_QMAX];
  for (int q = 0; q < Q; ++q) acc[q] = 0.0;
  const int k0 = kstart[j];
  for (int w = 0; w < W; ++w) {
    const int k = k0 + w;
    const int q = cls[(size_t)j * W + w];
    if (q < 0 || k < 0 || k >= n_per) continue;
    acc[q] += x[(size_t)b * n_per + k];
  }
  double s = 0.0;
  const size_t plane = (size_t)n_sk * nz;
  for (int q = 0; q < Q; ++q) {
    s = fma(taps[q], acc[q], s);
    R[q * plane + (size_t)b * nz + j] = s;
  }
}

// m[c nz + j] = sum over the skewers b near column c of P_cb R_b^(q_cb)[j]
// (z index j = threadIdx.x + t blockDim.x + blockIdx.y blockDim.x MC_PPT).
__global__ void k_mc_apply(int n_sk, int nz, const int* __restrict__ ptr,
                           const int* __restrict__ idx, const int* __restrict__ lev,
                           const double* __restrict__ p64, const double* __restrict__ R,
                           double* __restrict__ m, unsigned long long* prof_terms) {
  __shared__ size_t s_off[NB_CHUNK];
  __shared__ double s_p[NB_CHUNK];
  const int c = blockIdx.x;
  const int j0 = blockIdx.y * blockDim.x * MC_PPT + threadIdx.x;
  const int q0 = ptr[c], q1 = ptr[c + 1];
  double acc[MC_PPT];
  nbr_sum<double, MC_PPT, MC_U>(q0, q1, idx, lev, p64, -1, (size_t)n_sk * nz, nz, R, j0,
                                blockDim.x, nz, acc, s_off, s_p);
#pragma unroll
  for (int t = 0; t < MC_PPT; ++t) {
    const int j = j0 + t * blockDim.x;
    if (j < nz) m[(size_t)c * nz + j] = acc[t];
  }
  if (prof_terms && threadIdx.x == 0 && blockIdx.y == 0)
    atomicAdd(prof_terms, (unsigned long long)(q1 - q0) * nz);
}

// ---- neighbour lists (on the device) --------------------------------------------
// Target t (a skewer or a map column at (tx, ty)) and source skewer b are
// neighbours when c_perp |dxy|^2 + th[0] < cut; the entry keeps
// lev = #{q < Q : c_perp |dxy|^2 + th[q] < cut} (th ascending: the z part of
// the argument per level) and var_s exp(-c_perp |dxy|^2).  One warp per
// target scans the sources in order, so each row is in ascending b, and
// stores each entry's b and argument; k_list_finish then forms the levels
// and factors one thread per entry (in the scan, the FP64 work of the few
// lanes with an entry would hold the whole warp on GB300's FP64 pipe).
__global__ void k_list_count(int nt, const double* __restrict__ tx,
                             const double* __restrict__ ty, int ns,
                             const double* __restrict__ sx, const double* __restrict__ sy,
                             double c_perp, double lim, int* __restrict__ cnt) {
  const int t = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (t >= nt) return;
  int c = 0;
  for (int b = lane; b < ns; b += 32) {
    const double dx = tx[t] - sx[b], dy = ty[t] - sy[b];
    c += c_perp * (dx * dx + dy * dy) < lim;
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if (lane == 0) cnt[t] = c;
}

__global__ void k_list_fill(int nt, const double* __restrict__ tx, const double* __restrict__ ty,
                            int ns, const double* __restrict__ sx,
                            const double* __restrict__ sy, double c_perp, double cut,
                            const double* __restrict__ th, const int* __restrict__ ptr,
                            int* __restrict__ idx, double* __restrict__ p64) {
  const int t = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (t >= nt) return;
  int base = ptr[t];
  for (int b0 = 0; b0 < ns; b0 += 32) {
    const int b = b0 + lane;
    double parg = 0.0;
    bool ok = false;
    if (b < ns) {
      const double dx = tx[t] - sx[b], dy = ty[t] - sy[b];
      parg = c_perp * (dx * dx + dy * dy);
      ok = parg + th[0] < cut;
    }
    const unsigned m = __ballot_sync(0xffffffffu, ok);
    if (ok) {
      const int at = base + __popc(m & ((1u << lane) - 1u));
      idx[at] = b;
      p64[at] = parg;
    }
    base += __popc(m);
  }
}

// Entry e's level (the count of th[q] with arg + th[q] < cut: a binary
// search, the predicate falling with q) and factor, from its argument in p64.
__global__ void k_list_finish(long long n, double cut, double var_s, int Q,
                              const double* __restrict__ th, int* __restrict__ lev,
                              double* __restrict__ p64, float* __restrict__ p32) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const double parg = p64[e];
  int lo = 0, hi = Q;  // the count lies in [lo, hi]
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (parg + th[mid] < cut)
      lo = mid + 1;
    else
      hi = mid;
  }
  const double pv = var_s * exp(-parg);
  lev[e] = lo;
  p64[e] = pv;
  if (p32) p32[e] = (float)pv;
}

// Skewer (x, y) and skewer 0's z values, then a flag for any record not at
// its skewer's (x, y) or not at skewer 0's k-th z.
__global__ void k_sk_info(int n_sk, int n_per, const int* __restrict__ inv,
                          const double* __restrict__ px, const double* __restrict__ py,
                          const double* __restrict__ pz, double* __restrict__ sx,
                          double* __restrict__ sy, double* __restrict__ z) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n_sk) {
    const int p = inv[(size_t)i * n_per];
    sx[i] = px[p];
    sy[i] = py[p];
  }
  if (i < n_per) z[i] = pz[inv[i]];
}

__global__ void k_sk_check(size_t n, int n_per, const int* __restrict__ inv,
                           const double* __restrict__ px, const double* __restrict__ py,
                           const double* __restrict__ pz, const double* __restrict__ sx,
                           const double* __restrict__ sy, const double* __restrict__ z,
                           int* __restrict__ bad) {
  const size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int s = (int)(r / n_per), k = (int)(r % n_per);
  const int p = inv[r];
  if (px[p] != sx[s] || py[p] != sy[s] || pz[p] != z[k]) atomicOr(bad, 1);
}

}  // namespace

// CSR lists of targets against skewers for the z thresholds th[0..Q) (see
// k_list_fill); returns the number of entries.
static long long build_lists(int nt, const double* tx, const double* ty, int ns,
                             const double* sx, const double* sy, const KernelConsts& kc,
                             double cut, const std::vector<double>& th, DevBuf<int>& ptr,
                             DevBuf<int>& idx, DevBuf<int>& lev, DevBuf<double>& p64,
                             DevBuf<float>* p32, cudaStream_t st) {
  const int Q = (int)th.size();
  DevBuf<double> dth;
  DevBuf<int> cnt;
  dth.alloc(Q);
  cnt.alloc(nt);
  DS_CUDA(cudaMemcpyAsync(dth.p, th.data(), Q * sizeof(double), cudaMemcpyHostToDevice, st));
  const unsigned blocks = (unsigned)((nt + 7) / 8);  // 8 warps per CTA
  k_list_count<<<blocks, 256, 0, st>>>(nt, tx, ty, ns, sx, sy, kc.c_perp, cut - th[0], cnt.p);
  DS_CHECK_LAUNCH();
  std::vector<int> h(nt + 1, 0);
  DS_CUDA(cudaMemcpyAsync(h.data() + 1, cnt.p, nt * sizeof(int), cudaMemcpyDeviceToHost, st));
  DS_CUDA(cudaStreamSynchronize(st));
  for (int t = 0; t < nt; ++t) h[t + 1] += h[t];
  const long long total = h[nt];
  ptr.alloc(nt + 1);
  idx.alloc(std::max<long long>(1, total));
  lev.alloc(std::max<long long>(1, total));
  p64.alloc(std::max<long long>(1, total));
  if (p32) p32->alloc(std::max<long long>(1, total));
  DS_CUDA(cudaMemcpyAsync(ptr.p, h.data(), (nt + 1) * sizeof(int), cudaMemcpyHostToDevice, st));
  k_list_fill<<<blocks, 256, 0, st>>>(nt, tx, ty, ns, sx, sy, kc.c_perp, cut, dth.p, ptr.p,
                                      idx.p, p64.p);
  DS_CHECK_LAUNCH();
  if (total > 0) {
    k_list_finish<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(
        total, cut, kc.var_s, Q, dth.p, lev.p, p64.p, p32 ? p32->p : nullptr);
    DS_CHECK_LAUNCH();
  }
  DS_CUDA(cudaStreamSynchronize(st));  // h, dth, cnt go out of scope
  return total;
}

// Skewer pairs within `cut`: z thresholds c_para (z_m - z_0)^2 below cut.
static void build_nbrs(SkewerGrid& g, SkewerNbrs& nb, const KernelConsts& kc, double cut,
                       cudaStream_t st) {
  std::vector<double> th;
  for (int m = 0; m < g.n_per && kc.c_para * g.zd[m] * g.zd[m] < cut; ++m)
    th.push_back(kc.c_para * g.zd[m] * g.zd[m]);
  nb.cut = cut;
  nb.lmax = (int)th.size() - 1;  // the pair (a, a) keeps every level
  const long long total = build_lists(g.n_sk, g.sx.p, g.sy.p, g.n_sk, g.sx.p, g.sy.p, kc, cut,
                                      th, nb.ptr, nb.idx, nb.lev, nb.p64, &nb.p32, st);
  nb.n_terms = total * g.n_per;
}

namespace {

void build_skewer_grid(ds_operator* op, int n_sk, int n_per) {
  require(op->kc.eval == DS_EVAL_EXACT, "the structured operator needs the exact kernel");
  require(n_sk > 0 && n_per > 0 && n_per <= 1024 && (long long)n_sk * n_per == op->n,
          "n_skewers x n_per must equal the operator's record count (n_per <= 1024)");
  cudaStream_t st = op->ctx->stream;
  const size_t n = (size_t)op->n;
  std::unique_ptr<SkewerGrid, SkewerGridDeleter> g(new SkewerGrid());
  g->n_sk = n_sk;
  g->n_per = n_per;
  // every skewer at one (x, y), all on skewer 0's z values (checked on the device)
  DevBuf<double> dz;
  DevBuf<int> bad;
  g->sx.alloc(n_sk);
  g->sy.alloc(n_sk);
  dz.alloc(n_per);
  bad.alloc(1);
  DS_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), st));
  const int ni = std::max(n_sk, n_per);
  k_sk_info<<<(ni + 255) / 256, 256, 0, st>>>(n_sk, n_per, op->inv.p, op->pix.x.p, op->pix.y.p,
                                               op->pix.z.p, g->sx.p, g->sy.p, dz.p);
  DS_CHECK_LAUNCH();
  k_sk_check<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, n_per, op->inv.p, op->pix.x.p,
                                                           op->pix.y.p, op->pix.z.p, g->sx.p,
                                                           g->sy.p, dz.p, bad.p);
  DS_CHECK_LAUNCH();
  std::vector<double> z(n_per);
  int hbad = 0;
  DS_CUDA(cudaMemcpyAsync(z.data(), dz.p, n_per * sizeof(double), cudaMemcpyDeviceToHost, st));
  DS_CUDA(cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  DS_CUDA(cudaStreamSynchronize(st));
  require(!hbad, "structured operator: records must be skewers (one x, y each) on one z grid");
  // a uniform grid: (z_{k+m} - z_k) gives the same argument as z_m - z_0 to
  // 1e-13 (so each Toeplitz tap is the entry's own value to ~1e-13)
  std::vector<double> zd(n_per);
  for (int m = 0; m < n_per; ++m) zd[m] = z[m] - z[0];
  for (int k = 1; k < n_per; ++k) require(z[k] > z[k - 1], "structured operator: z not increasing");
  for (int m = 1; m < n_per; ++m) {
    const double want = op->kc.c_para * zd[m] * zd[m];
    if (want > op->kc.exact_cut) break;
    for (int k = 0; k + m < n_per; ++k) {
      const double d = z[k + m] - z[k];
      require(std::fabs(op->kc.c_para * d * d - want) <= 1e-13 * std::max(1.0, want),
              "structured operator: the z grid is not uniform");
    }
  }
  g->z0 = z[0];
  g->dz = n_per > 1 ? zd[1] : 0.0;
  g->zd = std::move(zd);
  std::vector<double> taps(n_per);
  std::vector<float> t32(n_per);
  for (int m = 0; m < n_per; ++m) {
    taps[m] = std::exp(-op->kc.c_para * g->zd[m] * g->zd[m]);
    t32[m] = (float)taps[m];
  }
  g->taps64.alloc(n_per);
  g->taps32.alloc(n_per);
  DS_CUDA(cudaMemcpyAsync(g->taps64.p, taps.data(), n_per * sizeof(double),
                          cudaMemcpyHostToDevice, st));
  DS_CUDA(cudaMemcpyAsync(g->taps32.p, t32.data(), n_per * sizeof(float),
                          cudaMemcpyHostToDevice, st));
  build_nbrs(*g, g->outer, op->kc, op->kc.exact_cut, st);
  g->V64.alloc((size_t)(g->outer.lmax + 1) * n);
  DS_CUDA(cudaStreamSynchronize(st));  // taps, t32 go out of scope
  op->sgrid = std::move(g);
}

}  // namespace

void skewer_apply_f64(ds_operator* op, const SkewerVecs& c, bool residual, const double* v,
                      double* out, const int* skip, cudaStream_t st) {
  SkewerGrid& g = *op->sgrid;
  const size_t n = (size_t)op->n;
  Profiler& pr = op->ctx->prof;
  cudaEvent_t ev = nullptr;
  unsigned long long* prof_terms = nullptr;
  if (pr.enabled) {
    prof_terms = pr.d_pairs;  // kind 0: FP64-accurate products and residuals
    pr.begin(st, &ev);
  }
  k_sg_levels<<<g.n_sk, g.n_per, g.n_per * sizeof(double), st>>>(
      g.n_per, g.outer.lmax, n, c.pos, c.wr, v, g.taps64.p, g.V64.p, skip);
  DS_CHECK_LAUNCH();
  const unsigned threads = (unsigned)((g.n_per + SG_PPT - 1) / SG_PPT);
  if (residual)
    k_sg_apply<true><<<g.n_sk, threads, 0, st>>>(g.n_per, n, g.outer.ptr.p, g.outer.idx.p,
                                                 g.outer.lev.p, g.outer.p64.p, g.V64.p, c.pos,
                                                 c.wl, c.e, v, c.b, out, skip, prof_terms);
  else
    k_sg_apply<false><<<g.n_sk, threads, 0, st>>>(g.n_per, n, g.outer.ptr.p, g.outer.idx.p,
                                                  g.outer.lev.p, g.outer.p64.p, g.V64.p, c.pos,
                                                  c.wl, c.e, v, c.b, out, skip, prof_terms);
  DS_CHECK_LAUNCH();
  if (ev) pr.end(st, ev, 0);
}

// Record-order copies of the operator's coefficients and right-hand side
// (record r at index r, padding 1 in pdiag and 0 elsewhere), for the mixed
// solve in record order.
__global__ void k_sg_rec_coeffs(int n, int n_pad, const int* __restrict__ inv,
                                const double* __restrict__ wl, const double* __restrict__ wr,
                                const double* __restrict__ e, const double* __restrict__ b,
                                const float* __restrict__ pd, double* __restrict__ rwl,
                                double* __restrict__ rwr, double* __restrict__ re,
                                double* __restrict__ rb, float* __restrict__ rpd) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_pad) return;
  if (r < n) {
    const int p = inv[r];
    rwl[r] = wl[p];
    rwr[r] = wr[p];
    re[r] = e[p];
    rb[r] = b[p];
    rpd[r] = pd[p];
  } else {
    rwl[r] = rwr[r] = re[r] = rb[r] = 0.0;
    rpd[r] = 1.f;
  }
}

__global__ void k_sg_to_rec(int n, int n_pad, const int* __restrict__ inv,
                            const double* __restrict__ sorted, double* __restrict__ rec) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n_pad) rec[r] = r < n ? sorted[inv[r]] : 0.0;
}

__global__ void k_sg_to_sorted(int n, const int* __restrict__ inv, const double* __restrict__ rec,
                               double* __restrict__ sorted) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n) sorted[inv[r]] = rec[r];
}

SkewerVecs skewer_vecs_rec(ds_operator* op, const float* pdiag_sorted) {
  SkewerGrid& g = *op->sgrid;
  const int np = op->pix.n_pad;
  if (!g.rb.p) {
    g.rwl.alloc(np);
    g.rwr.alloc(np);
    g.re.alloc(np);
    g.rb.alloc(np);
    g.rpd.alloc(np);
    g.rx.alloc(np);
    k_sg_rec_coeffs<<<(np + 255) / 256, 256, 0, op->ctx->stream>>>(
        op->n, np, op->inv.p, op->wl.p, op->wr.p, op->e.p, op->b.p, pdiag_sorted, g.rwl.p,
        g.rwr.p, g.re.p, g.rb.p, g.rpd.p);
    DS_CHECK_LAUNCH();
  }
  return SkewerVecs{nullptr, g.rwl.p, g.rwr.p, g.re.p, g.rb.p};
}

void skewer_x_to_rec(ds_operator* op, const double* x_sorted, double* x_rec, cudaStream_t st) {
  const int np = op->pix.n_pad;
  k_sg_to_rec<<<(np + 255) / 256, 256, 0, st>>>(op->n, np, op->inv.p, x_sorted, x_rec);
  DS_CHECK_LAUNCH();
}

void skewer_x_to_sorted(ds_operator* op, const double* x_rec, double* x_sorted, cudaStream_t st) {
  k_sg_to_sorted<<<(op->n + 255) / 256, 256, 0, st>>>(op->n, op->inv.p, x_rec, x_sorted);
  DS_CHECK_LAUNCH();
}

// Distance classes, pixel windows and column -> skewer lists of a column
// grid against the operator's skewer grid, for one cutoff.
// ---- fused float-pair map ------------------------------------------------------
// The same terms as k_mc_levels + k_mc_apply (pair (c, b) keeps the classes
// q < lev_cb of its z window) in a different order:
//   m[c, j] = sum_{k in window(j)} T_cls(j,k) Z_c^(cls(j,k))[k],
//   Z_c^(q)[k] = sum_{b: lev_cb > q} P_cb x_b[k],
// so each column needs its neighbours' pixel rows once (not their
// class-summed rows at every map z: 256 instead of 512 terms per pair on the
// 262,144-pixel workload).  With the list sorted by lev descending, one
// running sum over the list gives every Z^(q): when lev drops below q + 1,
// the sum so far is Z^(q).  All arithmetic is in float pairs (about 48
// significant bits; GB300 issues FP64 at 1/64 of FP32), rounded to FP64 once
// per output.
constexpr int MF_T = 256;  // threads per column
constexpr int MF_KMAX = 4; // pixels per thread at most (n_per <= 1024)
constexpr int MF_U = 8;    // neighbour rows in flight per thread

// Sorts each column's list by lev descending (stable by skewer), the factor
// split into a float pair.  One warp per column, a counting sort: the
// entries' levels counted 32 at a time, each level's first slot (levels
// descending, level 0 -- no class kept -- last), then each entry to its
// level's next slot, ranked within its 32 by the lanes of equal level below
// it (list order kept within a level).
constexpr int MC_SW = 8;  // columns (warps) per CTA of the sort
__global__ void __launch_bounds__(32 * MC_SW)
    k_mc_sort(int ncol, int Q, const int* __restrict__ ptr, const int* __restrict__ idx,
              const int* __restrict__ lev, const double* __restrict__ p64,
              int* __restrict__ sidx, int* __restrict__ slev, float2* __restrict__ sp) {
  __shared__ int s_next[MC_SW][MC_QMAX + 2];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * MC_SW + w;
  if (c >= ncol) return;  // the whole warp
  int* next = s_next[w];
  const int q0 = ptr[c], q1 = ptr[c + 1];
  for (int L = lane; L <= Q + 1; L += 32) next[L] = 0;
  __syncwarp();
  const unsigned below = (1u << lane) - 1u;
  for (int e0 = q0; e0 < q1; e0 += 32) {
    const int e = e0 + lane;
    int L = -1;  // no entry
    if (e < q1) {
      L = lev[e];
      if (L < 1 || L > Q) L = 0;
    }
    const unsigned same = __match_any_sync(0xffffffffu, L);
    if (L >= 0 && (same & below) == 0) next[L] += __popc(same);
    __syncwarp();
  }
  if (lane == 0) {
    int pos = q0;
    for (int L = Q; L >= 0; --L) {
      const int cnt = next[L];
      next[L] = pos;
      pos += cnt;
    }
  }
  __syncwarp();
  for (int e0 = q0; e0 < q1; e0 += 32) {
    const int e = e0 + lane;
    int L = -1;
    if (e < q1) {
      L = lev[e];
      if (L < 1 || L > Q) L = 0;
    }
    const unsigned same = __match_any_sync(0xffffffffu, L);
    if (L >= 0) {
      const int at = next[L] + __popc(same & below);
      if (L == 0) {  // contributes nothing
        sidx[at] = 0;
        slev[at] = 0;
        sp[at] = make_float2(0.f, 0.f);
      } else {
        const ff f = ff_from_double(p64[e]);
        sidx[at] = idx[e];
        slev[at] = L;
        sp[at] = make_float2(f.h, f.l);
      }
    }
    __syncwarp();
    if (L >= 0 && (same & below) == 0) next[L] += __popc(same);
    __syncwarp();
  }
}

// *acc += (*n_pairs) x per_pair (the profiler's term count).
__global__ void k_add_terms(unsigned long long* acc, const int* n_pairs,
                            unsigned long long per_pair) {
  atomicAdd(acc, (unsigned long long)*n_pairs * per_pair);
}

// x (FP64) as float pairs.
__global__ void k_mc_split(int n, const double* __restrict__ x, float2* __restrict__ xff) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const ff f = ff_from_double(x[i]);
    xff[i] = make_float2(f.h, f.l);
  }
}

// One CTA per map column: Z^(q) in shared memory (Q x n_per float pairs),
// then the window sums.  MF_K pixels per thread (MF_K MF_T >= n_per).
template <int MF_K>
__global__ void __launch_bounds__(MF_T) k_mc_fused(int nz, int n_per, int W, int Q,
                                                   const int* __restrict__ ptr,
                                                   const int* __restrict__ sidx,
                                                   const int* __restrict__ slev,
                                                   const float2* __restrict__ sp,
                                                   const float2* __restrict__ xff,
                                                   const int* __restrict__ kstart,
                                                   const signed char* __restrict__ cls,
                                                   const float2* __restrict__ taps,
                                                   double* __restrict__ m) {
  extern __shared__ float2 Zs[];  // Q x n_per
  __shared__ int s_off[MF_T];
  __shared__ int s_lev[MF_T];
  __shared__ float2 s_p[MF_T];
  const int c = blockIdx.x;
  const int tid = threadIdx.x;
  const int q0 = ptr[c], q1 = ptr[c + 1];
  ff S[MF_K];
#pragma unroll
  for (int t = 0; t < MF_K; ++t) S[t] = ff{0.f, 0.f};
  int lprev = Q;  // the same in every thread (all walk the same list)
  for (int c0 = q0; c0 < q1; c0 += MF_T) {
    const int cnt = min(MF_T, q1 - c0);
    __syncthreads();
    if (tid < cnt) {
      s_off[tid] = sidx[c0 + tid] * n_per;
      s_lev[tid] = slev[c0 + tid];
      s_p[tid] = sp[c0 + tid];
    }
    __syncthreads();
    for (int e0 = 0; e0 < cnt; e0 += MF_U) {
      float2 xv[MF_U][MF_K];
#pragma unroll
      for (int u = 0; u < MF_U; ++u)
#pragma unroll
        for (int t = 0; t < MF_K; ++t) {
          const int k = tid + t * MF_T;
          xv[u][t] = (e0 + u < cnt && k < n_per) ? __ldg(xff + s_off[e0 + u] + k)
                                                 : make_float2(0.f, 0.f);
        }
#pragma unroll
      for (int u = 0; u < MF_U; ++u) {
        if (e0 + u >= cnt) break;
        const int L = s_lev[e0 + u];
        if (L < lprev) {  // the sum so far is Z^(q) for q in [L, lprev)
          for (int q = L; q < lprev; ++q)
#pragma unroll
            for (int t = 0; t < MF_K; ++t) {
              const int k = tid + t * MF_T;
              if (k < n_per) Zs[q * n_per + k] = make_float2(S[t].h, S[t].l);
            }
          lprev = L;
        }
        const float2 pv = s_p[e0 + u];
#pragma unroll
        for (int t = 0; t < MF_K; ++t)
          ff_mac(S[t].h, S[t].l, ff{pv.x, pv.y}, ff{xv[u][t].x, xv[u][t].y});
      }
    }
  }
  for (int q = 0; q < lprev; ++q)
#pragma unroll
    for (int t = 0; t < MF_K; ++t) {
      const int k = tid + t * MF_T;
      if (k < n_per) Zs[q * n_per + k] = make_float2(S[t].h, S[t].l);
    }
  __syncthreads();
  for (int j = tid; j < nz; j += MF_T) {
    float ah = 0.f, al = 0.f;
    const int k0 = kstart[j];
    for (int w = 0; w < W; ++w) {
      const int q = cls[(size_t)j * W + w];
      const int k = k0 + w;
      if (q < 0 || k < 0 || k >= n_per) continue;
      const float2 z = Zs[q * n_per + k];
      const float2 tp = taps[q];
      ff_mac(ah, al, ff{tp.x, tp.y}, ff{z.x, z.y});
    }
    m[(size_t)c * nz + j] = (double)ah + (double)al;
  }
}

static void build_map_columns(ds_map* map, ds_operator* op, double cut) {
  MapColumns& mc = *map->cols;
  const SkewerGrid& g = *op->sgrid;
  const KernelConsts& kc = op->kc;
  cudaStream_t st = map->ctx->stream;
  const int nz = mc.nz, n_per = g.n_per;
  require(g.dz > 0.0, "structured map: the skewers need at least two pixels");
  const double dmax = std::sqrt(cut / kc.c_para);
  std::vector<int> kstart(nz);
  int W = 1;
  for (int j = 0; j < nz; ++j) {
    const int lo = (int)std::ceil((mc.z[j] - dmax - g.z0) / g.dz) - 1;
    const int hi = (int)std::floor((mc.z[j] + dmax - g.z0) / g.dz) + 1;
    kstart[j] = lo;
    W = std::max(W, hi - lo + 1);
  }
  auto dist = [&](int j, int k) { return std::fabs(mc.z[j] - (g.z0 + g.zd[k])); };
  std::vector<double> ds;
  for (int j = 0; j < nz; ++j)
    for (int w = 0; w < W; ++w) {
      const int k = kstart[j] + w;
      if (k < 0 || k >= n_per) continue;
      const double d = dist(j, k);
      if (kc.c_para * d * d < cut) ds.push_back(d);
    }
  // the distinct distances in ascending order (on grids of commensurate
  // spacing a few dozen: a sorted insertion; past 256, a sort of all), then
  // one representative per class, ulp-level ties merged (exact duplicates
  // never open a class, so dropping them first changes nothing)
  std::vector<double> du;
  for (double d : ds) {
    const auto it = std::lower_bound(du.begin(), du.end(), d);
    if (it != du.end() && *it == d) continue;
    if (du.size() >= 256) {
      du = ds;
      std::sort(du.begin(), du.end());
      break;
    }
    du.insert(it, d);
  }
  std::vector<double> cls_d;  // one representative per class
  for (double d : du)
    if (cls_d.empty() || d - cls_d.back() > 1e-12 * std::max(1.0, d)) cls_d.push_back(d);
  const int Q = (int)cls_d.size();
  require(Q >= 1 && Q <= MC_QMAX,
          "structured map: the map's z values and the pixels' z grid give more than 32 "
          "distances within the cutoff");
  auto class_of = [&](double d) {
    const auto it = std::lower_bound(cls_d.begin(), cls_d.end(), d * (1.0 - 1e-12) - 1e-300);
    return (int)(it - cls_d.begin());
  };
  std::vector<signed char> cls((size_t)nz * W, -1);
  for (int j = 0; j < nz; ++j)
    for (int w = 0; w < W; ++w) {
      const int k = kstart[j] + w;
      if (k < 0 || k >= n_per) continue;
      const double d = dist(j, k);
      if (kc.c_para * d * d < cut) cls[(size_t)j * W + w] = (signed char)class_of(d);
    }
  std::vector<double> taps(Q);
  for (int q = 0; q < Q; ++q) taps[q] = std::exp(-kc.c_para * cls_d[q] * cls_d[q]);
  // column -> skewer lists (z thresholds: the distance classes)
  std::vector<double> th(Q);
  for (int q = 0; q < Q; ++q) th[q] = kc.c_para * cls_d[q] * cls_d[q];
  build_lists(mc.ncol, mc.cx.p, mc.cy.p, g.n_sk, g.sx.p, g.sy.p, kc, cut, th, mc.ptr, mc.idx,
              mc.lev, mc.p64, nullptr, st);
  mc.Q = Q;
  mc.W = W;
  mc.cut = cut;
  mc.op_serial = op->serial;
  mc.kstart.alloc(nz);
  mc.cls.alloc(cls.size());
  mc.taps.alloc(Q);
  // the fused form's sorted lists and float-pair taps (R, the FP64 form's
  // class sums, is allocated when that form runs)
  mc.fidx.alloc(mc.idx.n);
  mc.flev.alloc(mc.idx.n);
  mc.fp.alloc(mc.idx.n);
  k_mc_sort<<<(mc.ncol + MC_SW - 1) / MC_SW, 32 * MC_SW, 0, st>>>(
      mc.ncol, Q, mc.ptr.p, mc.idx.p, mc.lev.p, mc.p64.p, mc.fidx.p, mc.flev.p, mc.fp.p);
  DS_CHECK_LAUNCH();
  std::vector<float2> ftaps(Q);
  for (int q = 0; q < Q; ++q) {
    const float h = (float)taps[q];
    ftaps[q] = make_float2(h, (float)(taps[q] - (double)h));
  }
  mc.ftaps.alloc(Q);
  DS_CUDA(cudaMemcpyAsync(mc.ftaps.p, ftaps.data(), Q * sizeof(float2), cudaMemcpyHostToDevice,
                          st));
  DS_CUDA(cudaMemcpyAsync(mc.kstart.p, kstart.data(), nz * sizeof(int), cudaMemcpyHostToDevice,
                          st));
  DS_CUDA(cudaMemcpyAsync(mc.cls.p, cls.data(), cls.size(), cudaMemcpyHostToDevice, st));
  DS_CUDA(cudaMemcpyAsync(mc.taps.p, taps.data(), Q * sizeof(double), cudaMemcpyHostToDevice,
                          st));
  DS_CUDA(cudaStreamSynchronize(st));  // host vectors go out of scope
}

bool skewer_map_product(ds_map* map, ds_operator* op, const double* x_dev, double* m_dev,
                        double cut) {
  if (!map->cols || !op->sgrid) return false;
  MapColumns& mc = *map->cols;
  if (mc.op_serial != op->serial || mc.cut != cut || !mc.ptr.p) build_map_columns(map, op, cut);
  const SkewerGrid& g = *op->sgrid;
  cudaStream_t st = map->ctx->stream;
  Profiler& pr = map->ctx->prof;
  cudaEvent_t ev = nullptr;
  unsigned long long* prof_terms = nullptr;
  if (pr.enabled) {
    prof_terms = pr.d_pairs + 2;  // kind 2: map products
    pr.begin(st, &ev);
  }
  // the fused float-pair form when a column's Z^(q) fit in shared memory
  const size_t zs_bytes = (size_t)mc.Q * g.n_per * sizeof(float2);
  static int smem_optin = -1;
  if (smem_optin < 0) {
    int dev = 0;
    DS_CUDA(cudaGetDevice(&dev));
    DS_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  }
  if (g.n_per <= MF_T * MF_KMAX && zs_bytes + 4 * 1024 <= (size_t)smem_optin) {
    const int K = (g.n_per + MF_T - 1) / MF_T;
    auto fn = K == 1 ? k_mc_fused<1> : K == 2 ? k_mc_fused<2> : K == 3 ? k_mc_fused<3>
                                                                         : k_mc_fused<4>;
    if (zs_bytes > 48 * 1024)
      DS_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)zs_bytes));
    const int n = g.n_sk * g.n_per;
    mc.xff.alloc(n);
    k_mc_split<<<std::min(1024, (n + 255) / 256), 256, 0, st>>>(n, x_dev, mc.xff.p);
    DS_CHECK_LAUNCH();
    fn<<<mc.ncol, MF_T, zs_bytes, st>>>(mc.nz, g.n_per, mc.W, mc.Q, mc.ptr.p, mc.fidx.p,
                                        mc.flev.p, mc.fp.p, mc.xff.p, mc.kstart.p, mc.cls.p,
                                        mc.ftaps.p, m_dev);
    DS_CHECK_LAUNCH();
    if (prof_terms) {  // the FP64 form's term count (pairs x map z), for comparable rates
      k_add_terms<<<1, 1, 0, st>>>(prof_terms, mc.ptr.p + mc.ncol, (unsigned long long)mc.nz);
      DS_CHECK_LAUNCH();
    }
  } else {
    mc.R.alloc((size_t)mc.Q * g.n_sk * mc.nz);
    k_mc_levels<<<dim3(g.n_sk, (mc.nz + 127) / 128), 128, 0, st>>>(
        g.n_sk, g.n_per, mc.nz, mc.W, mc.Q, mc.kstart.p, mc.cls.p, mc.taps.p, x_dev, mc.R.p);
    DS_CHECK_LAUNCH();
    k_mc_apply<<<dim3(mc.ncol, (mc.nz + 128 * MC_PPT - 1) / (128 * MC_PPT)), 128, 0, st>>>(
        g.n_sk, mc.nz, mc.ptr.p, mc.idx.p, mc.lev.p, mc.p64.p, mc.R.p, m_dev, prof_terms);
    DS_CHECK_LAUNCH();
  }
  if (ev) pr.end(st, ev, 2);
  return true;
}

void ensure_skewer_inner(ds_operator* op, double inner_cut) {
  SkewerGrid& g = *op->sgrid;
  if (g.inner.ptr.p && g.inner.cut == inner_cut) return;
  build_nbrs(g, g.inner, op->kc, inner_cut, op->ctx->stream);
  g.V32.alloc((size_t)(g.inner.lmax + 1) * op->n);
  g.dot_part.alloc(g.n_sk);
}

SkewerVecs skewer_vecs_sorted(ds_operator* op) {
  return SkewerVecs{op->inv.p, op->wl.p, op->wr.p, op->e.p, op->b.p};
}

void skewer_product_f32(ds_operator* op, const SkewerVecs& c, float* p, float* q,
                        unsigned int* counter, const double* num, double* alpha_out,
                        double* den_out, const int* skip, cudaStream_t st, const double* beta,
                        const float* z) {
  SkewerGrid& g = *op->sgrid;
  const size_t n = (size_t)op->n;
  Profiler& pr = op->ctx->prof;
  cudaEvent_t ev = nullptr;
  unsigned long long* prof_terms = nullptr;
  if (pr.enabled) {
    prof_terms = pr.d_pairs + 1;  // kind 1: FP32 products
    pr.begin(st, &ev);
  }
  k_sg32_levels<<<g.n_sk, g.n_per, g.n_per * sizeof(float), st>>>(
      g.n_per, g.inner.lmax, n, c.pos, c.wr, p, beta, z, g.taps32.p, g.V32.p, skip);
  DS_CHECK_LAUNCH();
  k_sg32_apply<<<g.n_sk, (g.n_per + SG_PPT - 1) / SG_PPT, 0, st>>>(
      g.n_per, n, g.inner.ptr.p, g.inner.idx.p, g.inner.lev.p, g.inner.p32.p, g.V32.p, c.pos,
      c.wl, c.e, p, q, counter ? g.dot_part.p : nullptr, counter, num, alpha_out, den_out, skip,
      prof_terms);
  DS_CHECK_LAUNCH();
  if (ev) pr.end(st, ev, 1);
}

}  // namespace ds

using namespace ds;

extern "C" {

int ds_operator_set_skewer_grid(ds_operator* op, int n_skewers, int n_per) {
  if (!op) return DS_ERR_ARG;
  return guarded(op->ctx, [&] {
    if (n_skewers == 0) {
      op->sgrid.reset();
      return;
    }
    build_skewer_grid(op, n_skewers, n_per);
  });
}

int ds_map_set_column_grid(ds_map* map, int n_columns, int nz) {
  if (!map) return DS_ERR_ARG;
  return guarded(map->ctx, [&] {
    if (n_columns == 0) {
      map->cols.reset();
      return;
    }
    require(n_columns > 0 && nz > 0 && (long long)n_columns * nz == map->n,
            "n_columns x nz must equal the map's point count");
    cudaStream_t st = map->ctx->stream;
    std::unique_ptr<MapColumns, MapColumnsDeleter> mc(new MapColumns());
    mc->ncol = n_columns;
    mc->nz = nz;
    mc->z.resize(nz);
    DevBuf<double> zj;
    DevBuf<int> bad;
    mc->cx.alloc(n_columns);
    mc->cy.alloc(n_columns);
    zj.alloc(nz);
    bad.alloc(1);
    DS_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), st));
    const int np = map->n;
    k_mc_info<<<(np + 255) / 256, 256, 0, st>>>(np, nz, map->raw.p, mc->cx.p, mc->cy.p, zj.p);
    DS_CHECK_LAUNCH();
    k_mc_check<<<(np + 255) / 256, 256, 0, st>>>(np, nz, map->raw.p, mc->cx.p, mc->cy.p, zj.p,
                                                  bad.p);
    DS_CHECK_LAUNCH();
    int hbad = 0;
    DS_CUDA(cudaMemcpyAsync(mc->z.data(), zj.p, nz * sizeof(double), cudaMemcpyDeviceToHost,
                            st));
    DS_CUDA(cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    DS_CUDA(cudaStreamSynchronize(st));
    require(!hbad, "map points are not a column grid (point c nz + j at column c's (x, y) "
                   "and the j-th z of column 0)");
    map->cols = std::move(mc);
  });
}

int ds_operator_skewer_product_dev(ds_operator* op, int residual, const double* v, double* out) {
  if (!op) return DS_ERR_ARG;
  return guarded(op->ctx, [&] {
    require(v && out, "null vector");
    require(op->sgrid != nullptr, "no skewer grid on this operator (ds_operator_set_skewer_grid)");
    cudaStream_t st = op->ctx->stream;
    op->tmp.alloc(op->pix.n_pad);
    op->tmp2.alloc(op->pix.n_pad);
    gather_sorted(op->pix, v, op->tmp.p, st);
    skewer_apply_f64(op, skewer_vecs_sorted(op), residual != 0, op->tmp.p, op->tmp2.p, nullptr,
                     st);
    scatter_sorted(op->pix, op->tmp2.p, nullptr, out, st);
  });
}

}  // extern "C"
