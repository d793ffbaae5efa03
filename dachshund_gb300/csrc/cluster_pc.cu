// Cluster preconditioner of the mixed-precision solver (no reference
// counterpart; the reference's PCG is Jacobi, lib/wf_vector.cc:42-49,185-194).
//
// Why clusters: the pixels of one skewer couple strongly along z, but a
// skewer also couples to its neighbours a few Mpc/h away, and on the skewer
// densities of these workloads that cross-skewer coupling is what Jacobi-PCG
// spends its iterations on.  Preconditioning each skewer's own 256 x 256
// block exactly (its full inverse) saves only a quarter of the iterations; a
// block over a cluster of four neighbouring skewers saves more than half.
//
// The factor: a factorized sparse approximate inverse (FSAI, Kolotilina and
// Yeremin 1993) of each cluster's block A_cc, in the order "by z, then by
// skewer" (the skewers' pixels interleaved), with a lower band of `band`
// sub-diagonals.  Column j of the lower-triangular G, on the rows
// J = j .. j + band of its cluster, is
//     g = A[J, J]^-1 e_1,   G[J, j] = g / sqrt(g_1),
// the band-limited counterpart of the Cholesky factor of A_cc^-1 (with the
// full pattern G G^T = A_cc^-1 exactly).  M^-1 = G G^T is symmetric positive
// definite by construction (G is triangular with a positive diagonal), and
// the solver applies it with the band kernel of mixed.cu (one CTA per
// cluster).  Each column is an independent (band + 1)-point Cholesky solve
// in FP32 from the operator's own coefficients, so the build is one short
// kernel; a column whose small system is not positive definite in FP32
// (none on the workloads here) falls back to the Jacobi factor 1/sqrt(A_jj).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <memory>
#include <numeric>
#include <vector>

#include "ds_device.cuh"
#include "ds_learned.h"
#include "ds_ops.h"

namespace ds {
namespace {

constexpr int CPC_MAX_BAND = 24;

// Column `j` (a slot) of G: rows j .. j + m - 1, the next non-padding slots
// of its block (at most band + 1).  A_ab = wl_a S_ab wr_b + e_a delta_ab with
// the exact Gaussian S evaluated in FP32 (the table kernel differs from it by
// ~1e-4, FP32 by ~1e-6: immaterial to a preconditioner).  One warp per
// column: lane a holds row a's coordinates and coefficients and forms row a
// of the system in shared memory; the Cholesky factor overwrites it column
// by column (lanes over the rows), then C y = e_1 (lanes over the rows) and
// C^T g = y (one row at a time); every entry takes the same operations in
// the same order as a one-thread-per-column solve, with the system in shared
// memory instead of 2 KB of per-thread stack.
constexpr int CPC_N = CPC_MAX_BAND + 1;  // rows of a column's system at most
constexpr int CPC_WARPS = 4;             // columns per CTA
__global__ void __launch_bounds__(32 * CPC_WARPS)
    k_cluster_fsai(int n_slots, int block, int band, KernelConsts kc, const int* __restrict__ crec,
                   const int* __restrict__ inv, const double* __restrict__ px,
                   const double* __restrict__ py, const double* __restrict__ pz,
                   const double* __restrict__ wl, const double* __restrict__ wr,
                   const double* __restrict__ e, float* __restrict__ L,
                   int* __restrict__ n_fallback) {
  __shared__ float sC[CPC_WARPS][CPC_N * CPC_N];  // row a at a CPC_N
  __shared__ float sy[CPC_WARPS][CPC_N];
  const int w = threadIdx.x >> 5, a = threadIdx.x & 31;
  const int j = blockIdx.x * CPC_WARPS + w;
  if (j >= n_slots || crec[j] < 0) return;  // the whole warp: padding slot (its row stays 0)
  float* C = sC[w];
  float* y = sy[w];
  const int blk_end = (j / block + 1) * block;
  const bool in = a <= band && j + a < blk_end && crec[j + a] >= 0;
  const unsigned out = __ballot_sync(0xffffffffu, !in);
  const int m = out ? __ffs(out) - 1 : 32;  // the first slot that is not a row ends them
  const int pa = a < m ? inv[crec[j + a]] : 0;
  const int p0 = __shfl_sync(0xffffffffu, pa, 0);
  // coordinates relative to the column's own pixel, in FP32 (a
  // preconditioner needs no more), and the coefficients of row a
  float rx = 0.f, ry = 0.f, rz = 0.f, wa = 0.f, wb = 0.f, ea = 0.f;
  if (a < m) {
    rx = (float)(px[pa] - px[p0]);
    ry = (float)(py[pa] - py[p0]);
    rz = (float)(pz[pa] - pz[p0]);
    wa = (float)(wl[pa] * kc.var_s);
    wb = (float)wr[pa];
    ea = (float)e[pa];
  }
  const float cp = (float)kc.c_perp, cq = (float)kc.c_para, cut = (float)kc.exact_cut;
  for (int b = 0; b < m; ++b) {
    const float xb = __shfl_sync(0xffffffffu, rx, b), yb = __shfl_sync(0xffffffffu, ry, b);
    const float zb = __shfl_sync(0xffffffffu, rz, b), wbb = __shfl_sync(0xffffffffu, wb, b);
    if (a < m && b <= a) {
      const float dx = rx - xb, dy = ry - yb, dz = rz - zb;
      const float arg = fmaf(cp, fmaf(dx, dx, dy * dy), cq * dz * dz);
      float v = arg < cut ? wa * expf(-arg) * wbb : 0.f;
      if (a == b) v += ea;
      C[a * CPC_N + b] = v;
    }
  }
  __syncwarp();
  // lower Cholesky factor, column b by lanes a >= b
  bool ok = true;
  for (int b = 0; b < m; ++b) {
    float v = 0.f;
    if (a >= b && a < m) {
      v = C[a * CPC_N + b];
      for (int k = 0; k < b; ++k) v = fmaf(-C[a * CPC_N + k], C[b * CPC_N + k], v);
    }
    const float d = __shfl_sync(0xffffffffu, v, b);
    if (!(d > 0.f)) {
      ok = false;
      break;
    }
    const float cbb = sqrtf(d);
    __syncwarp();
    if (a == b)
      C[a * CPC_N + a] = cbb;
    else if (a > b && a < m)
      C[a * CPC_N + b] = v / cbb;
    __syncwarp();
  }
  if (!ok) {
    if (a == 0) {
      const double a00 = wl[p0] * kc.var_s * wr[p0] + e[p0];
      L[j] = (float)(1.0 / sqrt(a00));  // plane 0: the diagonal
      atomicAdd(n_fallback, 1);
    }
    return;
  }
  // C y = e_1: lane a finishes y_a once y_0 .. y_{a-1} are known
  float yv = a == 0 ? 1.f : 0.f;
  for (int k = 0; k < m; ++k) {
    if (a == k) yv = yv / C[k * CPC_N + k];
    const float yk = __shfl_sync(0xffffffffu, yv, k);
    if (a > k && a < m) yv = fmaf(-C[a * CPC_N + k], yk, yv);
  }
  if (a < m) y[a] = yv;
  __syncwarp();
  // C^T g = y (g overwrites y), from the last row up
  for (int r = m - 1; r >= 0; --r) {
    if (a == r) {
      float v = y[r];
      for (int k = r + 1; k < m; ++k) v = fmaf(-C[k * CPC_N + r], y[k], v);
      y[r] = v / C[r * CPC_N + r];
    }
    __syncwarp();
  }
  // G[j + a][j] is plane a at slot j + a
  if (a < m) L[(size_t)a * n_slots + (j + a)] = y[a] * rsqrtf(y[0]);
}

// The same column solve for bands up to MB - 1, one thread per column, every
// loop unrolled: the factor stays in registers (MB (MB + 1) / 2 floats),
// the rows' coordinates and coefficients in shared memory (row a of thread
// t at [c][a][t]), with the same operations in the same order as the warp
// form (measured on the 262,144-pixel workload: the warp form 0.98 ms, its
// lanes idle in the serial steps; one thread per column with the factor on
// a 2 KB stack, ~600 MB live at full occupancy, 0.57 ms).
constexpr int CPC_T = 64;  // columns per CTA of the unrolled form
template <int MB>
__global__ void __launch_bounds__(CPC_T)
    k_cluster_fsai_unrolled(int n_slots, int block, int band, KernelConsts kc,
                            const int* __restrict__ crec, const int* __restrict__ inv,
                            const double* __restrict__ px, const double* __restrict__ py,
                            const double* __restrict__ pz, const double* __restrict__ wl,
                            const double* __restrict__ wr, const double* __restrict__ e,
                            float* __restrict__ L, int* __restrict__ n_fallback) {
  __shared__ float sc[6][MB][CPC_T];  // rx, ry, rz, wa, wb, ea
  const int t = threadIdx.x;
  const int j = blockIdx.x * CPC_T + t;
  if (j >= n_slots || crec[j] < 0) return;  // padding slot: its row stays 0
  const int blk_end = (j / block + 1) * block;
  const int p0 = inv[crec[j]];
  const double x0 = px[p0], y0 = py[p0], z0 = pz[p0];
  int m = 0;  // the next non-padding slots of the block, at most band + 1
#pragma unroll
  for (int a = 0; a < MB; ++a)
    if (a == m && a <= band && j + a < blk_end && crec[j + a] >= 0) {
      const int pa = inv[crec[j + a]];
      sc[0][a][t] = (float)(px[pa] - x0);
      sc[1][a][t] = (float)(py[pa] - y0);
      sc[2][a][t] = (float)(pz[pa] - z0);
      sc[3][a][t] = (float)(wl[pa] * kc.var_s);
      sc[4][a][t] = (float)wr[pa];
      sc[5][a][t] = (float)e[pa];
      ++m;
    }
  const float cp = (float)kc.c_perp, cq = (float)kc.c_para, cut = (float)kc.exact_cut;
  float C[MB * (MB + 1) / 2];  // packed lower Cholesky factor: row a starts at a (a + 1) / 2
  bool ok = true;
#pragma unroll
  for (int a = 0; a < MB; ++a) {
    if (a >= m) break;
    const float xa = sc[0][a][t], ya = sc[1][a][t], za = sc[2][a][t];
    const float wa = sc[3][a][t], ea = sc[5][a][t];
#pragma unroll
    for (int b = 0; b <= a; ++b) {
      const float dx = xa - sc[0][b][t], dy = ya - sc[1][b][t], dz = za - sc[2][b][t];
      const float arg = fmaf(cp, fmaf(dx, dx, dy * dy), cq * dz * dz);
      float v = arg < cut ? wa * expf(-arg) * sc[4][b][t] : 0.f;
      if (a == b) v += ea;
#pragma unroll
      for (int k = 0; k < b; ++k) v = fmaf(-C[a * (a + 1) / 2 + k], C[b * (b + 1) / 2 + k], v);
      if (a == b) {
        ok = ok && v > 0.f;
        C[a * (a + 1) / 2 + a] = sqrtf(v);
      } else {
        C[a * (a + 1) / 2 + b] = v / C[b * (b + 1) / 2 + b];
      }
    }
  }
  if (!ok) {
    const double a00 = wl[p0] * kc.var_s * wr[p0] + e[p0];
    L[j] = (float)(1.0 / sqrt(a00));  // plane 0: the diagonal
    atomicAdd(n_fallback, 1);
    return;
  }
  // C y = e_1, then C^T g = y (g overwrites y)
  float y[MB];
#pragma unroll
  for (int a = 0; a < MB; ++a) {
    if (a >= m) break;
    float v = a == 0 ? 1.f : 0.f;
#pragma unroll
    for (int k = 0; k < a; ++k) v = fmaf(-C[a * (a + 1) / 2 + k], y[k], v);
    y[a] = v / C[a * (a + 1) / 2 + a];
  }
#pragma unroll
  for (int a = MB - 1; a >= 0; --a) {
    if (a >= m) continue;
    float v = y[a];
#pragma unroll
    for (int k = a + 1; k < MB; ++k)
      if (k < m) v = fmaf(-C[k * (k + 1) / 2 + a], y[k], v);
    y[a] = v / C[a * (a + 1) / 2 + a];
  }
  // G[j + a][j] is plane a at slot j + a
  const float scale = rsqrtf(y[0]);
#pragma unroll
  for (int a = 0; a < MB; ++a)
    if (a < m) L[(size_t)a * n_slots + (j + a)] = y[a] * scale;
}

// Record r's z, and skewer s's (x, y) from its first record (r = s n_per).
__global__ void k_rec_coords(int n, int n_per, const int* __restrict__ inv,
                             const double* __restrict__ px, const double* __restrict__ py,
                             const double* __restrict__ pz, double* __restrict__ sx,
                             double* __restrict__ sy, double* __restrict__ rz) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int p = inv[r];
  rz[r] = pz[p];
  if (r % n_per == 0) {
    sx[r / n_per] = px[p];
    sy[r / n_per] = py[p];
  }
}

// *bad = 1 unless every record's z equals skewer 0's z at the same pixel and
// skewer 0's z values increase (the shared z grid of plan_skewer_clusters).
__global__ void k_shared_z(int n, int n_per, const double* __restrict__ rz, int* __restrict__ bad) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int k = r % n_per;
  if (rz[r] != rz[k] || (r < n_per && k > 0 && !(rz[k - 1] < rz[k]))) atomicOr(bad, 1);
}

// The slots of the shared z grid: a cluster of sz skewers (the first sz of
// its g) holds pixel k of its j-th skewer at slot k sz + j, then -1 up to
// g n_per.
__global__ void k_crec_shared(int n_slots, int n_per, int g, const int* __restrict__ bsk,
                              int* __restrict__ crec) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_slots) return;
  const int B = g * n_per;
  const int c = i / B, o = i - c * B;
  const int* sk = bsk + (size_t)c * g;
  int sz = 0;
  while (sz < g && sk[sz] >= 0) ++sz;
  int v = -1;
  if (o < sz * n_per) {
    const int k = o / sz, j = o - k * sz;
    v = sk[j] * n_per + k;
  }
  crec[i] = v;
}

// 32-bit Morton key of (x, y) quantised to 16 bits each.
uint32_t morton2(uint32_t x, uint32_t y) {
  auto spread = [](uint32_t v) {
    v &= 0xFFFFu;
    v = (v | (v << 8)) & 0x00FF00FFu;
    v = (v | (v << 4)) & 0x0F0F0F0Fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
  };
  return spread(x) | (spread(y) << 1);
}

// Clusters of `g` neighbouring skewers and the slot order within each: the
// skewers are visited in Morton order of their (x, y); each unassigned one
// seeds a cluster with its g - 1 nearest unassigned skewers among the next
// 256 unassigned in that order.  A cluster's slots hold its records sorted by
// z, then by skewer; each block of g n_per slots is padded with -1.  With
// every skewer on skewer 0's increasing z values (`shared`) that order is
// pixel-major and crec is left empty (built on the device); otherwise rz
// holds every record's z.
void plan_skewer_clusters(int n_sk, int n_per, int g, const std::vector<double>& sx,
                          const std::vector<double>& sy, bool shared,
                          const std::vector<double>& rz, std::vector<int>& crec,
                          std::vector<int>& bsk, int& n_blocks) {
  const double x0 = *std::min_element(sx.begin(), sx.end());
  const double x1 = *std::max_element(sx.begin(), sx.end());
  const double y0 = *std::min_element(sy.begin(), sy.end());
  const double y1 = *std::max_element(sy.begin(), sy.end());
  const double span = std::max({x1 - x0, y1 - y0, 1e-300});
  std::vector<uint32_t> key(n_sk);
  for (int s = 0; s < n_sk; ++s)
    key[s] = morton2((uint32_t)std::lround((sx[s] - x0) / span * 65535.0),
                     (uint32_t)std::lround((sy[s] - y0) / span * 65535.0));
  std::vector<int> order(n_sk);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key[a] < key[b]; });
  constexpr int WINDOW = 256;
  std::vector<char> used(n_sk, 0);
  std::vector<std::vector<int>> clusters;
  const int kmax = g - 1;
  std::vector<std::pair<double, int>> best(std::max(1, kmax));
  for (int oi = 0; oi < n_sk; ++oi) {
    const int s0 = order[oi];
    if (used[s0]) continue;
    used[s0] = 1;
    // the g - 1 nearest by (squared distance, skewer index), ascending: an
    // insertion into the g - 1 best so far
    int take = 0;
    for (int oj = oi + 1, seen = 0; kmax > 0 && oj < n_sk && seen < WINDOW; ++oj) {
      const int s = order[oj];
      if (used[s]) continue;
      ++seen;
      const double dx = sx[s] - sx[s0], dy = sy[s] - sy[s0];
      const std::pair<double, int> p{dx * dx + dy * dy, s};
      if (take == kmax && !(p < best[kmax - 1])) continue;
      int at = take < kmax ? take++ : kmax - 1;
      while (at > 0 && p < best[at - 1]) {
        best[at] = best[at - 1];
        --at;
      }
      best[at] = p;
    }
    std::vector<int> c{s0};
    for (int k = 0; k < take; ++k) {
      c.push_back(best[k].second);
      used[best[k].second] = 1;
    }
    clusters.push_back(std::move(c));
  }
  n_blocks = (int)clusters.size();
  bsk.assign((size_t)n_blocks * g, -1);
  for (int c = 0; c < n_blocks; ++c)
    std::copy(clusters[c].begin(), clusters[c].end(), bsk.begin() + (size_t)c * g);
  if (shared) return;  // pixel-major: k_crec_shared
  const int B = g * n_per;
  crec.assign((size_t)n_blocks * B, -1);
  std::vector<int> recs;
  for (int c = 0; c < n_blocks; ++c) {
    recs.clear();
    for (int q : clusters[c])
      for (int k = 0; k < n_per; ++k) recs.push_back(q * n_per + k);
    // by z, then by the skewer's rank in the cluster (stable)
    std::stable_sort(recs.begin(), recs.end(), [&](int a, int b) { return rz[a] < rz[b]; });
    std::copy(recs.begin(), recs.end(), crec.begin() + (size_t)c * B);
  }
}

void build_cluster_pc(ds_operator* op, int n_sk, int n_per, int g, int band) {
  cudaStream_t st = op->ctx->stream;
  const int n = op->n;
  // skewer (x, y) (of each skewer's first record) and every record's z
  DevBuf<double> dsx, dsy, drz;
  dsx.alloc(n_sk);
  dsy.alloc(n_sk);
  drz.alloc(n);
  k_rec_coords<<<(n + 255) / 256, 256, 0, st>>>(n, n_per, op->inv.p, op->pix.x.p, op->pix.y.p,
                                                op->pix.z.p, dsx.p, dsy.p, drz.p);
  DS_CHECK_LAUNCH();
  DevBuf<int> dbad;
  dbad.alloc(1);
  DS_CUDA(cudaMemsetAsync(dbad.p, 0, sizeof(int), st));
  k_shared_z<<<(n + 255) / 256, 256, 0, st>>>(n, n_per, drz.p, dbad.p);
  DS_CHECK_LAUNCH();
  std::vector<double> sx(n_sk), sy(n_sk), rz;
  int bad = 0;
  DS_CUDA(cudaMemcpyAsync(sx.data(), dsx.p, n_sk * sizeof(double), cudaMemcpyDeviceToHost, st));
  DS_CUDA(cudaMemcpyAsync(sy.data(), dsy.p, n_sk * sizeof(double), cudaMemcpyDeviceToHost, st));
  DS_CUDA(cudaMemcpyAsync(&bad, dbad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  DS_CUDA(cudaStreamSynchronize(st));
  if (bad) {  // records off the shared z grid: the host orders each cluster by z
    rz.resize(n);
    DS_CUDA(cudaMemcpyAsync(rz.data(), drz.p, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    DS_CUDA(cudaStreamSynchronize(st));
  }
  std::vector<int> crec, bsk;
  int n_blocks = 0;
  plan_skewer_clusters(n_sk, n_per, g, sx, sy, !bad, rz, crec, bsk, n_blocks);

  std::unique_ptr<SkewerPC, SkewerPCDeleter> pc(new SkewerPC());
  pc->n_sk = n_blocks;
  pc->n_per = g * n_per;
  pc->band = band;
  const size_t n_slots = (size_t)n_blocks * g * n_per;
  pc->crec.alloc(n_slots);
  pc->L.alloc(n_slots * (band + 1));
  DevBuf<int> nfb;
  nfb.alloc(1);
  pc->g = g;
  pc->bsk.alloc(bsk.size());
  DS_CUDA(cudaMemcpyAsync(pc->bsk.p, bsk.data(), bsk.size() * sizeof(int),
                          cudaMemcpyHostToDevice, st));
  if (crec.empty()) {
    k_crec_shared<<<(unsigned)((n_slots + 255) / 256), 256, 0, st>>>((int)n_slots, n_per, g,
                                                                     pc->bsk.p, pc->crec.p);
    DS_CHECK_LAUNCH();
  } else {
    DS_CUDA(cudaMemcpyAsync(pc->crec.p, crec.data(), n_slots * sizeof(int),
                            cudaMemcpyHostToDevice, st));
  }
  DS_CUDA(cudaMemsetAsync(pc->L.p, 0, pc->L.bytes(), st));
  DS_CUDA(cudaMemsetAsync(nfb.p, 0, sizeof(int), st));
  if (band <= 16)
    k_cluster_fsai_unrolled<17><<<(unsigned)((n_slots + CPC_T - 1) / CPC_T), CPC_T, 0, st>>>(
        (int)n_slots, pc->n_per, band, op->kc, pc->crec.p, op->inv.p, op->pix.x.p, op->pix.y.p,
        op->pix.z.p, op->wl.p, op->wr.p, op->e.p, pc->L.p, nfb.p);
  else
    k_cluster_fsai<<<(unsigned)((n_slots + CPC_WARPS - 1) / CPC_WARPS), 32 * CPC_WARPS, 0, st>>>(
        (int)n_slots, pc->n_per, band, op->kc, pc->crec.p, op->inv.p, op->pix.x.p, op->pix.y.p,
        op->pix.z.p, op->wl.p, op->wr.p, op->e.p, pc->L.p, nfb.p);
  DS_CHECK_LAUNCH();
  DS_CUDA(cudaMemcpyAsync(&pc->n_fallback, nfb.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  DS_CUDA(cudaStreamSynchronize(st));
  op->pc = std::move(pc);
}

}  // namespace
}  // namespace ds

using namespace ds;

extern "C" {

int ds_operator_set_cluster_preconditioner(ds_operator* op, int n_skewers, int n_per,
                                           int cluster, int band, int* n_fallback) {
  if (!op) return DS_ERR_ARG;
  return guarded(op->ctx, [&] {
    if (cluster == 0) {
      op->pc.reset();
      return;
    }
    require(n_skewers > 0 && n_per > 0 && (long long)n_skewers * n_per == op->n,
            "n_skewers x n_per must equal the operator's record count");
    require(cluster > 0 && (long long)cluster * n_per <= 1024,
            "cluster x n_per must be in [1, 1024]");
    require(band >= 0 && band <= CPC_MAX_BAND, "band must be in [0, 24]");
    build_cluster_pc(op, n_skewers, n_per, cluster, band);
    if (n_fallback) *n_fallback = op->pc->n_fallback;
  });
}

}  // extern "C"
