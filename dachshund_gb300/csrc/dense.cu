// Dense paths: the operator A built densely in HBM, the dense FP64 matvec
// used by PCG when the matrix fits, the closed-form solve (Cholesky) that
// stands in for WFVector{SN,W}::solve_cf (lib/wf_vector.cc:123-155, 276-319),
// and MapCovarDiag (lib/map_covar.cc:40-113) as one SN-form solve per map
// point.
//
// Dense matvec: one warp per row, A streamed once per matvec (8 n^2 bytes)
// with evict-first loads, the vector read through L2.  Its bound on GB300 is
// the FP64 pipe (n^2 FMAs at 2/clk/SM, ~5 TB/s of matrix data) just below HBM
// (~6.8 TB/s).
// Cholesky: right-looking, 32-wide panels: diagonal block in shared memory by
// one CTA, the panel by a triangular solve per row, the trailing lower
// triangle by 64 x 64 tiles (each thread a 4 x 4 block).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "ds_device.cuh"
#include "ds_ops.h"

namespace ds {
namespace {

constexpr int NB = 32;       // Cholesky panel width
constexpr int DTILE = 64;    // trailing-update tile
constexpr int DW = 8;        // warps per CTA in the dense matvec

// A_ij of the operator for every (i, j) < n (row-major, leading dim ld), in
// the order of the given coordinate/coefficient arrays (sorted or caller).
__global__ void k_dense_build(KernelConsts kc, int n, size_t ld, const double* __restrict__ x,
                              const double* __restrict__ y, const double* __restrict__ z,
                              const double* __restrict__ wl, const double* __restrict__ e,
                              const double* __restrict__ table, double* __restrict__ A) {
  __shared__ double tf[TABLE_N];
  for (int k = threadIdx.x; k < TABLE_N; k += blockDim.x) tf[k] = table[k];
  __syncthreads();
  const size_t total = (size_t)n * n;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < total;
       q += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(q / n), j = (int)(q % n);
    const double dx = x[i] - x[j], dy = y[i] - y[j], dz = z[i] - z[j];
    double S;
    if (kc.eval == DS_EVAL_TABLE) {
      S = s_table_f64(dx, dy, dz, kc, tf);
    } else {
      const double arg = kc.c_perp * (dx * dx + dy * dy) + kc.c_para * (dz * dz);
      S = arg < kc.exact_cut ? kc.var_s * exp(-arg) : 0.0;
    }
    A[(size_t)i * ld + j] = wl[i] * S * wl[j] + (i == j ? e[i] : 0.0);
  }
}

// q = A v (+ last-CTA alpha = delta / (dotv . q)) or r = b - A v.
template <bool RESIDUAL, bool DOT>
__global__ void __launch_bounds__(DW * 32) k_dense_matvec(int n, size_t ld,
                                                         const double* __restrict__ A,
                                                         const double* __restrict__ v,
                                                         const double* __restrict__ b,
                                                         double* __restrict__ out,
                                                         const double* __restrict__ dotv,
                                                         double* part, PcgState* pcg,
                                                         unsigned int* counter,
                                                         const int* skip_flag,
                                                         unsigned long long* prof_pairs) {
  if (skip_flag && *skip_flag) return;
  if (prof_pairs && blockIdx.x == 0 && threadIdx.x == 0)
    atomicAdd(prof_pairs, (unsigned long long)n * (unsigned long long)n);
  __shared__ double red[DW];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int row = blockIdx.x * DW + w;
  double dot = 0.0;
  if (row < n) {
    const double* a = A + (size_t)row * ld;
    double acc = 0.0;
    int j = 2 * lane;
    for (; j + 1 < n; j += 64) {
      const double2 av = __ldcs(reinterpret_cast<const double2*>(a + j));
      acc = fma(av.x, v[j], acc);
      acc = fma(av.y, v[j + 1], acc);
    }
    if (j < n) acc = fma(__ldcs(a + j), v[j], acc);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) {
      const double o = RESIDUAL ? b[row] - acc : acc;
      out[row] = o;
      if (DOT) dot = dotv[row] * o;
    }
  }
  if (!DOT) return;
  if (lane == 0) red[w] = dot;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < DW; ++k) s += red[k];
    part[blockIdx.x] = s;
  }
  __shared__ double red2[DW];
  if (last_block_arrive(counter)) {
    const double dq = reduce_partials<DW * 32>(part, gridDim.x, 1, 0, red2);
    if (threadIdx.x == 0) {
      pcg->dq = dq;
      pcg->alpha = pcg->delta / dq;
      *counter = 0;
    }
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

// Map-covariance helpers: b_k = S(map_i, pix_k) (sorted pixel order; zero on
// padding) and sigma = b . x.
__global__ void k_map_column(KernelConsts kc, int n_pad, const int* __restrict__ perm,
                             const double* __restrict__ px, const double* __restrict__ py,
                             const double* __restrict__ pz, double mx, double my, double mz,
                             const double* __restrict__ table, double* __restrict__ b) {
  __shared__ double tf[TABLE_N];
  for (int k = threadIdx.x; k < TABLE_N; k += blockDim.x) tf[k] = table[k];
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_pad) return;
  b[i] = perm[i] >= 0 ? s_eval_f64<DS_EVAL_TABLE>(mx - px[i], my - py[i], mz - pz[i], kc, tf)
                      : 0.0;
}

__global__ void k_map_column_exact(KernelConsts kc, int n_pad, const int* __restrict__ perm,
                                   const double* __restrict__ px, const double* __restrict__ py,
                                   const double* __restrict__ pz, double mx, double my,
                                   double mz, double* __restrict__ b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_pad) return;
  const double dx = mx - px[i], dy = my - py[i], dz = mz - pz[i];
  b[i] = perm[i] >= 0 ? kc.var_s * exp(-(kc.c_perp * (dx * dx + dy * dy) + kc.c_para * dz * dz))
                      : 0.0;
}

__global__ void k_dot2(int n, const double* __restrict__ a, const double* __restrict__ b,
                       const double* __restrict__ c, double* out) {
  // out[0] = a.b, out[1] = c.c  (one CTA, deterministic)
  __shared__ double red[8];
  double s = 0.0, t = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    s = fma(a[i], b[i], s);
    t = fma(c[i], c[i], t);
  }
  const double bs = block_sum<256>(s, red);
  const double bt = block_sum<256>(t, red);
  if (threadIdx.x == 0) {
    out[0] = bs;
    out[1] = bt;
  }
}

}  // namespace

// ---- dense operator for PCG ------------------------------------------------

void op_build_dense(ds_operator* op) {
  cudaStream_t st = op->ctx->stream;
  const size_t np = op->pix.n_pad;
  op->dense.alloc(np * np);
  k_dense_build<<<4 * 152 * 8, 256, 0, st>>>(op->kc, (int)np, np, op->pix.x.p, op->pix.y.p,
                                              op->pix.z.p, op->wl.p, op->e.p, op->table.p,
                                              op->dense.p);
  DS_CHECK_LAUNCH();
  DS_CUDA(cudaStreamSynchronize(st));
}

void dense_apply(ds_operator* op, bool residual, const double* v, double* out,
                 const double* dotv, double* part, PcgState* pcg, unsigned int* counter,
                 const int* skip, cudaStream_t st) {
  const int np = op->pix.n_pad;
  const int grid = (np + DW - 1) / DW;
  Profiler& prof = op->ctx->prof;
  cudaEvent_t ev = nullptr;
  unsigned long long* pp = nullptr;
  if (prof.enabled) {
    pp = prof.d_pairs;
    prof.begin(st, &ev);
  }
  if (residual)
    k_dense_matvec<true, false><<<grid, DW * 32, 0, st>>>(np, np, op->dense.p, v, op->b.p, out,
                                                          nullptr, nullptr, nullptr, nullptr,
                                                          skip, pp);
  else if (dotv)
    k_dense_matvec<false, true><<<grid, DW * 32, 0, st>>>(np, np, op->dense.p, v, nullptr, out,
                                                          dotv, part, pcg, counter, skip, pp);
  else
    k_dense_matvec<false, false><<<grid, DW * 32, 0, st>>>(np, np, op->dense.p, v, nullptr, out,
                                                           nullptr, nullptr, nullptr, nullptr,
                                                           skip, pp);
  DS_CHECK_LAUNCH();
  if (ev) prof.end(st, ev, 0);
}

int dense_partials(int n_pad) { return (n_pad + DW - 1) / DW; }

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
  k_dense_build<<<4 * 152 * 8, 256, 0, st>>>(kc, n, n, x.p, y.p, z.p, wl.p, e.p, d_table, A.p);
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

// ---- MapCovarDiag ---------------------------------------------------------------

void map_covar_diag_run(ds_operator* op, int n_map, const double* map_pts,
                        const ds_pcg_params& pp, double* sigma_m, int* iters, int* success) {
  cudaStream_t st = op->ctx->stream;
  ensure_pcg_workspace(op);
  const int np = op->pix.n_pad;
  DevBuf<double> out2;
  out2.alloc(2);
  for (int i = 0; i < n_map; ++i) {
    const double* m = map_pts + (size_t)i * 3;
    if (op->kc.eval == DS_EVAL_TABLE)
      k_map_column<<<(np + 255) / 256, 256, 0, st>>>(op->kc, np, op->pix.perm.p, op->pix.x.p,
                                                     op->pix.y.p, op->pix.z.p, m[0], m[1], m[2],
                                                     op->table.p, op->b.p);
    else
      k_map_column_exact<<<(np + 255) / 256, 256, 0, st>>>(op->kc, np, op->pix.perm.p,
                                                           op->pix.x.p, op->pix.y.p, op->pix.z.p,
                                                           m[0], m[1], m[2], op->b.p);
    DS_CHECK_LAUNCH();
    DS_CUDA(cudaMemsetAsync(op->x.p, 0, np * sizeof(double), st));
    k_dot2<<<1, 256, 0, st>>>(np, op->b.p, op->x.p, op->b.p, out2.p);
    DS_CHECK_LAUNCH();
    double h2[2];
    DS_CUDA(cudaMemcpyAsync(h2, out2.p, sizeof(h2), cudaMemcpyDeviceToHost, st));
    DS_CUDA(cudaStreamSynchronize(st));
    op->norm_b = std::sqrt(h2[1]);
    ds_pcg_result r{};
    if (op->norm_b > 0.0) run_pcg(op, pp, r, nullptr);
    double s = 0.0;
    if (r.success) {
      k_dot2<<<1, 256, 0, st>>>(np, op->b.p, op->x.p, op->b.p, out2.p);
      DS_CHECK_LAUNCH();
      DS_CUDA(cudaMemcpyAsync(h2, out2.p, sizeof(h2), cudaMemcpyDeviceToHost, st));
      DS_CUDA(cudaStreamSynchronize(st));
      s = h2[0];
    }
    sigma_m[i] = s;
    iters[i] = r.num_iters;
    success[i] = r.success;
  }
}

}  // namespace ds
