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
#include "ds_ops.h"
#include "ds_skewer.h"

namespace ds {

void SkewerGridDeleter::operator()(SkewerGrid* p) const { delete p; }

namespace {

// V^(L) for L = 0..lmax of one skewer per CTA (n_per threads).
__global__ void k_sg_levels(int n_per, int lmax, size_t n, const int* __restrict__ pos,
                            const double* __restrict__ wr, const double* __restrict__ v,
                            const double* __restrict__ taps, double* __restrict__ V,
                            const int* skip) {
  if (skip && *skip) return;
  extern __shared__ double su[];
  const int k = threadIdx.x;
  const size_t r = (size_t)blockIdx.x * n_per + k;
  const int p = pos[r];
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
template <bool RESID>
__global__ void k_sg_apply(int n_per, size_t n, const int* __restrict__ nb_ptr,
                           const int* __restrict__ nb_idx, const int* __restrict__ nb_lev,
                           const double* __restrict__ nb_p, const double* __restrict__ V,
                           const int* __restrict__ pos, const double* __restrict__ wl,
                           const double* __restrict__ e, const double* __restrict__ v,
                           const double* __restrict__ bvec, double* __restrict__ out,
                           const int* skip, unsigned long long* prof_terms) {
  if (skip && *skip) return;
  const int a = blockIdx.x, k = threadIdx.x;
  const int q0 = nb_ptr[a], q1 = nb_ptr[a + 1];
  double acc0 = 0.0, acc1 = 0.0;
  int q = q0;
  for (; q + 1 < q1; q += 2) {  // two independent chains
    const double v0 = V[(size_t)nb_lev[q] * n + (size_t)nb_idx[q] * n_per + k];
    const double v1 = V[(size_t)nb_lev[q + 1] * n + (size_t)nb_idx[q + 1] * n_per + k];
    acc0 = fma(nb_p[q], v0, acc0);
    acc1 = fma(nb_p[q + 1], v1, acc1);
  }
  if (q < q1)
    acc0 = fma(nb_p[q], V[(size_t)nb_lev[q] * n + (size_t)nb_idx[q] * n_per + k], acc0);
  const size_t r = (size_t)a * n_per + k;
  const int p = pos[r];
  const double y = fma(wl[p], acc0 + acc1, e[p] * v[p]);
  out[p] = RESID ? bvec[p] - y : y;
  if (prof_terms && k == 0) atomicAdd(prof_terms, (unsigned long long)(q1 - q0) * n_per);
}

// FP32 levels of the inner operator: u = wr p (FP32 vectors, sorted order).
__global__ void k_sg32_levels(int n_per, int lmax, size_t n, const int* __restrict__ pos,
                              const double* __restrict__ wr, const float* __restrict__ p,
                              const float* __restrict__ taps, float* __restrict__ V,
                              const int* skip) {
  if (skip && *skip) return;
  extern __shared__ float sf[];
  const int k = threadIdx.x;
  const size_t r = (size_t)blockIdx.x * n_per + k;
  const int ps = pos[r];
  const float u = (float)wr[ps] * p[ps];
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
  const int a = blockIdx.x, k = threadIdx.x;
  const int q0 = nb_ptr[a], q1 = nb_ptr[a + 1];
  float acc0 = 0.f, acc1 = 0.f;
  int j = q0;
  for (; j + 1 < q1; j += 2) {
    const float v0 = V[(size_t)nb_lev[j] * n + (size_t)nb_idx[j] * n_per + k];
    const float v1 = V[(size_t)nb_lev[j + 1] * n + (size_t)nb_idx[j + 1] * n_per + k];
    acc0 = fmaf(nb_p[j], v0, acc0);
    acc1 = fmaf(nb_p[j + 1], v1, acc1);
  }
  if (j < q1)
    acc0 = fmaf(nb_p[j], V[(size_t)nb_lev[j] * n + (size_t)nb_idx[j] * n_per + k], acc0);
  const size_t r = (size_t)a * n_per + k;
  const int ps = pos[r];
  const float pv = p[ps];
  const float qv = fmaf((float)wl[ps], acc0 + acc1, (float)e[ps] * pv);
  q[ps] = qv;
  if (prof_terms && k == 0) atomicAdd(prof_terms, (unsigned long long)(q1 - q0) * n_per);
  if (!part) return;
  const double s = sg_cta_sum((double)pv * (double)qv, sm);
  if (k == 0) part[a] = s;
  if (!last_block_arrive(counter)) return;
  double t = 0.0;
  for (int c = k; c < (int)gridDim.x; c += blockDim.x) t += __ldcg(part + c);
  const double pq = sg_cta_sum(t, sm);
  if (k == 0) {
    *den_out = pq;
    *alpha_out = *num / pq;
    *counter = 0;
  }
}

// Skewer pairs within `cut` (cell lists of side sqrt(cut / c_perp)).
void build_nbrs(SkewerNbrs& nb, const std::vector<double>& sx, const std::vector<double>& sy,
                const std::vector<double>& zd, const KernelConsts& kc, double cut, int n_per,
                cudaStream_t st) {
  const int n_sk = (int)sx.size();
  nb.cut = cut;
  const double h = std::sqrt(cut / kc.c_perp);
  const double x0 = *std::min_element(sx.begin(), sx.end());
  const double y0 = *std::min_element(sy.begin(), sy.end());
  const double x1 = *std::max_element(sx.begin(), sx.end());
  const double y1 = *std::max_element(sy.begin(), sy.end());
  const int ncx = std::max(1, (int)std::min(4096.0, std::floor((x1 - x0) / h) + 1));
  const int ncy = std::max(1, (int)std::min(4096.0, std::floor((y1 - y0) / h) + 1));
  auto cell_of = [&](double v, double o, int nc) {
    return std::min(nc - 1, std::max(0, (int)std::floor((v - o) / h)));
  };
  std::vector<std::vector<int>> cells((size_t)ncx * ncy);
  for (int s = 0; s < n_sk; ++s)
    cells[(size_t)cell_of(sy[s], y0, ncy) * ncx + cell_of(sx[s], x0, ncx)].push_back(s);
  std::vector<int> ptr(n_sk + 1, 0), idx, lev;
  std::vector<double> p64;
  std::vector<std::pair<int, double>> row;
  nb.lmax = 0;
  nb.n_terms = 0;
  for (int a = 0; a < n_sk; ++a) {
    const int cx = cell_of(sx[a], x0, ncx), cy = cell_of(sy[a], y0, ncy);
    row.clear();
    for (int jy = std::max(0, cy - 1); jy <= std::min(ncy - 1, cy + 1); ++jy)
      for (int jx = std::max(0, cx - 1); jx <= std::min(ncx - 1, cx + 1); ++jx)
        for (int b : cells[(size_t)jy * ncx + jx]) {
          const double dx = sx[a] - sx[b], dy = sy[a] - sy[b];
          const double parg = kc.c_perp * (dx * dx + dy * dy);
          if (parg < cut) row.push_back({b, parg});
        }
    std::sort(row.begin(), row.end());
    for (const auto& bp : row) {
      int L = 0;
      while (L + 1 < n_per && bp.second + kc.c_para * (zd[L + 1] * zd[L + 1]) < cut) ++L;
      idx.push_back(bp.first);
      lev.push_back(L);
      p64.push_back(kc.var_s * std::exp(-bp.second));
      nb.lmax = std::max(nb.lmax, L);
    }
    ptr[a + 1] = (int)idx.size();
    nb.n_terms += (long long)row.size() * n_per;
  }
  nb.ptr.alloc(ptr.size());
  nb.idx.alloc(std::max<size_t>(1, idx.size()));
  nb.lev.alloc(std::max<size_t>(1, lev.size()));
  nb.p64.alloc(std::max<size_t>(1, p64.size()));
  DS_CUDA(cudaMemcpyAsync(nb.ptr.p, ptr.data(), ptr.size() * sizeof(int), cudaMemcpyHostToDevice,
                          st));
  DS_CUDA(cudaMemcpyAsync(nb.idx.p, idx.data(), idx.size() * sizeof(int), cudaMemcpyHostToDevice,
                          st));
  DS_CUDA(cudaMemcpyAsync(nb.lev.p, lev.data(), lev.size() * sizeof(int), cudaMemcpyHostToDevice,
                          st));
  DS_CUDA(cudaMemcpyAsync(nb.p64.p, p64.data(), p64.size() * sizeof(double),
                          cudaMemcpyHostToDevice, st));
  std::vector<float> p32(p64.begin(), p64.end());
  nb.p32.alloc(std::max<size_t>(1, p32.size()));
  DS_CUDA(cudaMemcpyAsync(nb.p32.p, p32.data(), p32.size() * sizeof(float),
                          cudaMemcpyHostToDevice, st));
  DS_CUDA(cudaStreamSynchronize(st));  // host vectors go out of scope
}

void build_skewer_grid(ds_operator* op, int n_sk, int n_per) {
  require(op->kc.eval == DS_EVAL_EXACT, "the structured operator needs the exact kernel");
  require(n_sk > 0 && n_per > 0 && n_per <= 1024 && (long long)n_sk * n_per == op->n,
          "n_skewers x n_per must equal the operator's record count (n_per <= 1024)");
  cudaStream_t st = op->ctx->stream;
  const int n = op->n, np = op->pix.n_pad;
  std::vector<double> hx(np), hy(np), hz(np);
  std::vector<int> hinv(n);
  DS_CUDA(cudaMemcpyAsync(hx.data(), op->pix.x.p, np * sizeof(double),
                          cudaMemcpyDeviceToHost, st));
  DS_CUDA(cudaMemcpyAsync(hy.data(), op->pix.y.p, np * sizeof(double),
                          cudaMemcpyDeviceToHost, st));
  DS_CUDA(cudaMemcpyAsync(hz.data(), op->pix.z.p, np * sizeof(double),
                          cudaMemcpyDeviceToHost, st));
  DS_CUDA(cudaMemcpyAsync(hinv.data(), op->inv.p, n * sizeof(int), cudaMemcpyDeviceToHost, st));
  DS_CUDA(cudaStreamSynchronize(st));
  // every skewer at one (x, y), all on skewer 0's z values
  std::vector<double> sx(n_sk), sy(n_sk), z(n_per);
  for (int k = 0; k < n_per; ++k) z[k] = hz[hinv[k]];
  for (int s = 0; s < n_sk; ++s) {
    const int p0 = hinv[(size_t)s * n_per];
    sx[s] = hx[p0];
    sy[s] = hy[p0];
    for (int k = 0; k < n_per; ++k) {
      const int p = hinv[(size_t)s * n_per + k];
      require(hx[p] == sx[s] && hy[p] == sy[s] && hz[p] == z[k],
              "structured operator: records must be skewers (one x, y each) on one z grid");
    }
  }
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
  std::unique_ptr<SkewerGrid, SkewerGridDeleter> g(new SkewerGrid());
  g->n_sk = n_sk;
  g->n_per = n_per;
  g->dz = n_per > 1 ? zd[1] : 0.0;
  std::vector<double> taps(n_per);
  for (int m = 0; m < n_per; ++m) taps[m] = std::exp(-op->kc.c_para * zd[m] * zd[m]);
  g->taps64.alloc(n_per);
  DS_CUDA(cudaMemcpyAsync(g->taps64.p, taps.data(), n_per * sizeof(double),
                          cudaMemcpyHostToDevice, st));
  build_nbrs(g->outer, sx, sy, zd, op->kc, op->kc.exact_cut, n_per, st);
  g->V64.alloc((size_t)(g->outer.lmax + 1) * n);
  std::vector<float> t32(taps.begin(), taps.end());
  g->taps32.alloc(n_per);
  DS_CUDA(cudaMemcpyAsync(g->taps32.p, t32.data(), n_per * sizeof(float),
                          cudaMemcpyHostToDevice, st));
  DS_CUDA(cudaStreamSynchronize(st));
  g->sx = std::move(sx);
  g->sy = std::move(sy);
  g->zd = std::move(zd);
  op->sgrid = std::move(g);
}

}  // namespace

void skewer_apply_f64(ds_operator* op, bool residual, const double* v, double* out,
                      const int* skip, cudaStream_t st) {
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
      g.n_per, g.outer.lmax, n, op->inv.p, op->wr.p, v, g.taps64.p, g.V64.p, skip);
  DS_CHECK_LAUNCH();
  if (residual)
    k_sg_apply<true><<<g.n_sk, g.n_per, 0, st>>>(g.n_per, n, g.outer.ptr.p, g.outer.idx.p,
                                                 g.outer.lev.p, g.outer.p64.p, g.V64.p,
                                                 op->inv.p, op->wl.p, op->e.p, v, op->b.p, out,
                                                 skip, prof_terms);
  else
    k_sg_apply<false><<<g.n_sk, g.n_per, 0, st>>>(g.n_per, n, g.outer.ptr.p, g.outer.idx.p,
                                                  g.outer.lev.p, g.outer.p64.p, g.V64.p,
                                                  op->inv.p, op->wl.p, op->e.p, v, op->b.p, out,
                                                  skip, prof_terms);
  DS_CHECK_LAUNCH();
  if (ev) pr.end(st, ev, 0);
}

void ensure_skewer_inner(ds_operator* op, double inner_cut) {
  SkewerGrid& g = *op->sgrid;
  if (g.inner.ptr.p && g.inner.cut == inner_cut) return;
  build_nbrs(g.inner, g.sx, g.sy, g.zd, op->kc, inner_cut, g.n_per, op->ctx->stream);
  g.V32.alloc((size_t)(g.inner.lmax + 1) * op->n);
  g.dot_part.alloc(g.n_sk);
}

void skewer_product_f32(ds_operator* op, const float* p, float* q, unsigned int* counter,
                        const double* num, double* alpha_out, double* den_out,
                        const int* skip, cudaStream_t st) {
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
      g.n_per, g.inner.lmax, n, op->inv.p, op->wr.p, p, g.taps32.p, g.V32.p, skip);
  DS_CHECK_LAUNCH();
  k_sg32_apply<<<g.n_sk, g.n_per, 0, st>>>(g.n_per, n, g.inner.ptr.p, g.inner.idx.p,
                                           g.inner.lev.p, g.inner.p32.p, g.V32.p, op->inv.p,
                                           op->wl.p, op->e.p, p, q,
                                           counter ? g.dot_part.p : nullptr, counter, num,
                                           alpha_out, den_out, skip, prof_terms);
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

int ds_operator_skewer_product_dev(ds_operator* op, int residual, const double* v, double* out) {
  if (!op) return DS_ERR_ARG;
  return guarded(op->ctx, [&] {
    require(v && out, "null vector");
    require(op->sgrid != nullptr, "no skewer grid on this operator (ds_operator_set_skewer_grid)");
    cudaStream_t st = op->ctx->stream;
    op->tmp.alloc(op->pix.n_pad);
    op->tmp2.alloc(op->pix.n_pad);
    gather_sorted(op->pix, v, op->tmp.p, st);
    skewer_apply_f64(op, residual != 0, op->tmp.p, op->tmp2.p, nullptr, st);
    scatter_sorted(op->pix, op->tmp2.p, nullptr, out, st);
  });
}

}  // extern "C"
