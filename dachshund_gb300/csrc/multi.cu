// MapCovarDiag (lib/map_covar.cc:40-113) with the reference's table kernel
// as a multi-right-hand-side FP64 Jacobi-PCG.
//
// The reference solves (S + N) x = S_pm[:, i] from x = 0 once per map point
// i, sequentially, and takes sigma_m[i] = S_mp[i, :] . x.  Every solve uses
// the same operator, so here MR map points are solved together: the pair
// kernel evaluates each table-kernel value S_jk once and applies it to the MR
// vectors (~17 FP64 instructions for the kernel value + MR FMAs per pair,
// against 17 + 1 per pair and right-hand side for separate solves), and each
// right-hand side keeps its own CG scalars, convergence test and iteration
// count, so every map point follows the reference's recurrence
// (lib/pcg.h:27-160): the same preconditioner, a full residual every step_r
// iterations, |r| <= tol |b|, the same iteration-count and success rules.  A
// right-hand side that has converged is frozen; the launches of an iteration
// return at once when all have.
//
// Vectors are n_pad x R doubles in the operator's sorted order with the
// right-hand side fastest (v[i * R + r]), R a power of two from 16 to 256.
// Reductions are deterministic (fixed tree and partial orders, no floating
// atomics).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "ds_device.cuh"
#include "ds_ops.h"

namespace ds {
namespace {

constexpr int MR = 16;       // right-hand sides per CTA of the pair kernel
constexpr int MR_MAX = 256;  // right-hand sides per solve at most
constexpr int MVB = 256;     // threads per vector-kernel CTA (R divides it)
constexpr int MVGRID = 304;  // vector-kernel CTAs at most
constexpr int MCHECK = 8;    // iterations between host reads of the done flag

struct MState {  // one right-hand side
  double delta, delta_old, alpha, beta, dq, norm_r, norm_b, tol_norm_b;
  int iter, done, converged, pad;
};

struct MShared {
  int all_done;
  int max_iter;
  int R;  // right-hand sides of this solve
  int pad;
  unsigned int counter[4];
};

struct MPairArgs {
  const double *rx, *ry, *rz;
  const int *row_ptr, *cols, *row_order;
  const unsigned short* mask;
  const double *wl, *wr, *e, *table;
  const double* v;     // n_pad x R
  const double* b;     // n_pad x R (residual)
  double* out;         // n_pad x R
  const double* dotv;  // n_pad x R (fused dots)
  double* part;        // n_row_tiles x R
  MState* st;
  MShared* sh;
};

inline int mgrid(size_t n) {
  return (int)std::max<size_t>(1, std::min<size_t>(MVGRID, (n + MVB - 1) / MVB));
}

// q = A v for R vectors (+ per right-hand side d.q -> alpha by the last
// CTA) or r = b - A v, with the operator's table kernel and coefficients.
// CTA (x, y): row tile x (heaviest first) and right-hand sides [16 y, 16 y +
// 16); one row per thread, a warp's column sub-tiles staged warp-privately
// as in the single-vector FP64 kernel.
template <bool RESID, bool DOT>
__global__ void __launch_bounds__(TILE) k_mpair(KernelConsts kc, MPairArgs a) {
  if (a.sh->all_done) return;
  __shared__ double sxyz[TILE / 32][3][SUBTILE];
  __shared__ __align__(16) double su[TILE / 32][SUBTILE][MR];
  __shared__ double tf[TABLE_N];
  __shared__ double red[TILE / 32][MR];
  __shared__ int live;
  __shared__ bool last;
  const int R = a.sh->R, r0 = blockIdx.y * MR;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // a block whose 16 right-hand sides have all converged has nothing to do
  // (with DOT it still arrives, so that the last CTA finds every partial)
  if (tid == 0) {
    int l = 0;
    for (int r = 0; r < MR; ++r) l |= !a.st[r0 + r].done;
    live = l;
  }
  __syncthreads();
  if (!live && !DOT) return;
  if (live) {
    const int t = a.row_order ? a.row_order[blockIdx.x] : blockIdx.x;
    const int i = t * TILE + tid;
    for (int k = tid; k < TABLE_N; k += TILE) tf[k] = a.table[k];
    __syncthreads();
    const double xi = a.rx[i], yi = a.ry[i], zi = a.rz[i];
    double acc[MR];
#pragma unroll
    for (int r = 0; r < MR; ++r) acc[r] = 0.0;
    const int p0 = a.row_ptr[t], p1 = a.row_ptr[t + 1];
    for (int p = p0; p < p1; ++p) {
      const unsigned m = (a.mask[p] >> (4 * warp)) & 0xFu;  // this warp's row sub-tile
      if (!m) continue;
      const int ct = a.cols[p];
      for (int cs = 0; cs < TILE / SUBTILE; ++cs) {
        if (!((m >> cs) & 1u)) continue;
        const int j = ct * TILE + cs * SUBTILE + lane;
        __syncwarp();
        sxyz[warp][0][lane] = a.rx[j];
        sxyz[warp][1][lane] = a.ry[j];
        sxyz[warp][2][lane] = a.rz[j];
        const double wj = kc.var_s * a.wr[j];
        const double2* vj = reinterpret_cast<const double2*>(a.v + (size_t)j * R + r0);
#pragma unroll
        for (int r2 = 0; r2 < MR / 2; ++r2) {
          const double2 q = vj[r2];
          su[warp][lane][2 * r2] = wj * q.x;
          su[warp][lane][2 * r2 + 1] = wj * q.y;
        }
        __syncwarp();
        for (int jj = 0; jj < SUBTILE; ++jj) {
          const double g = gp_table_fast(xi - sxyz[warp][0][jj], yi - sxyz[warp][1][jj],
                                         zi - sxyz[warp][2][jj], kc, tf);
          const double2* uj = reinterpret_cast<const double2*>(su[warp][jj]);
#pragma unroll
          for (int r2 = 0; r2 < MR / 2; ++r2) {
            const double2 u = uj[r2];
            acc[2 * r2] = fma(g, u.x, acc[2 * r2]);
            acc[2 * r2 + 1] = fma(g, u.y, acc[2 * r2 + 1]);
          }
        }
      }
    }
    const double wli = a.wl[i], ei = a.e[i];
    double dots[MR];
#pragma unroll
    for (int r = 0; r < MR; ++r) {
      const size_t k = (size_t)i * R + r0 + r;
      const double q = wli * acc[r] + ei * a.v[k];
      const double o = RESID ? a.b[k] - q : q;
      if (!a.st[r0 + r].done) a.out[k] = o;  // a converged right-hand side stays as it was
      dots[r] = DOT ? a.dotv[k] * o : 0.0;
    }
    if (!DOT) return;
    // per right-hand side: warp trees, then the four warps in order
#pragma unroll
    for (int r = 0; r < MR; ++r) {
      double v = dots[r];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0) red[warp][r] = v;
    }
    __syncthreads();
    if (tid < MR)
      a.part[(size_t)blockIdx.x * R + r0 + tid] =
          (red[0][tid] + red[1][tid]) + (red[2][tid] + red[3][tid]);
  } else if (tid < MR) {
    a.part[(size_t)blockIdx.x * R + r0 + tid] = 0.0;
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) last = atomicAdd(&a.sh->counter[0], 1u) == gridDim.x * gridDim.y - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  // the last CTA: d.q per right-hand side over all row tiles, in tile order
  for (int r = tid; r < R; r += TILE) {
    double dq = 0.0;
    for (int k = 0; k < (int)gridDim.x; ++k) dq += __ldcg(a.part + (size_t)k * R + r);
    MState& st = a.st[r];
    if (!st.done) {
      st.dq = dq;
      st.alpha = st.delta / dq;  // lib/pcg.h:37
    }
  }
  if (tid == 0) a.sh->counter[0] = 0;
}

// Per right-hand side sums over the grid of two values each thread holds
// for r = threadIdx.x % R (R divides the block and the grid stride); the
// last CTA gets them in tot[0..R) and tot[R..2R).  Fixed order: the block's
// threads of one r in index order, then the CTAs in order.
__device__ __forceinline__ bool grid_sum_by_rhs(int R, double v0, double v1, double* part,
                                                unsigned int* counter, double* tot) {
  __shared__ double sm[2][MVB];
  __shared__ bool last;
  sm[0][threadIdx.x] = v0;
  sm[1][threadIdx.x] = v1;
  __syncthreads();
  for (int idx = threadIdx.x; idx < 2 * R; idx += MVB) {  // 2 R may exceed the block
    const int c = idx / R, r = idx % R;
    double s = 0.0;
    for (int k = r; k < MVB; k += R) s += sm[c][k];
    part[(size_t)blockIdx.x * 2 * R + idx] = s;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return false;
  __threadfence();
  for (int c = threadIdx.x; c < 2 * R; c += MVB) {
    double s = 0.0;
    for (int k = 0; k < (int)gridDim.x; ++k) s += __ldcg(part + (size_t)k * 2 * R + c);
    tot[c] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) *counter = 0;
  return true;
}

// |b| per right-hand side, the tolerance, and the right-hand sides with
// |b| <= 0 marked done (lib/pcg.h:79-86: they return early, unsuccessful).
__global__ void __launch_bounds__(MVB) k_mnorm(size_t n, const double* __restrict__ b,
                                               double tol, MState* st, MShared* sh,
                                               double* part) {
  __shared__ double tot[2 * MR_MAX];
  const int R = sh->R;
  double bb = 0.0;
  for (size_t e = (size_t)blockIdx.x * MVB + threadIdx.x; e < n; e += (size_t)gridDim.x * MVB)
    bb = fma(b[e], b[e], bb);
  if (!grid_sum_by_rhs(R, bb, 0.0, part, &sh->counter[1], tot)) return;
  for (int r = threadIdx.x; r < R; r += MVB) {
    MState& s = st[r];
    s.norm_b = sqrt(tot[r]);
    s.tol_norm_b = tol * s.norm_b;  // lib/pcg.h:93
    s.iter = 0;
    s.converged = 0;
    s.done = s.norm_b > 0.0 ? 0 : 1;
    s.alpha = s.beta = s.dq = s.norm_r = 0.0;
  }
}

// mode 0: normal step (x, r recurrences + precondition + dots)
// mode 1: x update only (full-residual step, before the residual kernel)
// mode 2: precondition + dots only (full-residual step, after the residual)
// mode 3: start from x = 0: r = b, d = M^-1 r + dots
template <int MODE>
__global__ void __launch_bounds__(MVB) k_mupdate(size_t n, MState* st, MShared* sh,
                                                 double* __restrict__ x, double* __restrict__ r,
                                                 double* __restrict__ d,
                                                 const double* __restrict__ q,
                                                 double* __restrict__ s,
                                                 const double* __restrict__ b,
                                                 const double* __restrict__ pdiag,
                                                 double* part, double* hist, int hist_stride) {
  if (MODE != 3 && sh->all_done) return;
  __shared__ double tot[2 * MR_MAX];
  const int R = sh->R;
  const int rr = threadIdx.x % R;  // this thread's right-hand side (R divides the stride)
  const bool live = !st[rr].done;
  const double alpha = st[rr].alpha;
  double rs = 0.0, r2 = 0.0;
  for (size_t e = (size_t)blockIdx.x * MVB + threadIdx.x; e < n; e += (size_t)gridDim.x * MVB) {
    if (!live) break;
    if (MODE == 0 || MODE == 1) x[e] = fma(alpha, d[e], x[e]);  // lib/pcg.h:39
    if (MODE == 1) continue;
    double ri;
    if (MODE == 3) {
      ri = b[e];  // r = b - A x with x = 0
      r[e] = ri;
    } else {
      ri = r[e];
    }
    if (MODE == 0) {
      ri = fma(-alpha, q[e], ri);  // lib/pcg.h:48
      r[e] = ri;
    }
    const double si = ri / pdiag[e / R];  // lib/pcg.h:52
    s[e] = si;
    if (MODE == 3) d[e] = si;
    rs = fma(ri, si, rs);
    r2 = fma(ri, ri, r2);
  }
  if (MODE == 1) return;
  if (!grid_sum_by_rhs(R, rs, r2, part, &sh->counter[1], tot)) return;
  for (int rq = threadIdx.x; rq < R; rq += MVB) {
    MState& S = st[rq];
    const double trs = tot[rq], trr = tot[R + rq];
    double* h = hist + (size_t)rq * hist_stride;
    if (MODE == 3) {
      if (!S.done) {
        S.delta = trs;  // lib/pcg.h:104
        S.norm_r = sqrt(trr);
        h[0] = S.norm_r;
        if (sh->max_iter <= 1) S.done = 1;
      }
    } else if (!S.done) {
      S.delta_old = S.delta;
      S.delta = trs;                        // lib/pcg.h:58
      S.beta = S.delta / S.delta_old;       // lib/pcg.h:61
      const int it = S.iter + 1;
      S.iter = it;
      S.norm_r = sqrt(trr);                 // lib/pcg.h:123-126
      h[it] = S.norm_r;
      if (S.norm_r <= S.tol_norm_b) {       // lib/pcg.h:130
        S.done = 1;
        S.converged = 1;
      } else if (it + 1 >= sh->max_iter) {  // loop exit, lib/pcg.h:118,151
        S.done = 1;
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int all = 1;
    for (int k = 0; k < R; ++k) all &= st[k].done;
    sh->all_done = all;
  }
}

// d = s + beta d (lib/pcg.h:62-64) for the right-hand sides still running.
__global__ void __launch_bounds__(MVB) k_mdir(size_t n, const MState* st, const MShared* sh,
                                              const double* __restrict__ s,
                                              double* __restrict__ d) {
  if (sh->all_done) return;
  const int rr = threadIdx.x % sh->R;
  if (st[rr].done) return;
  const double beta = st[rr].beta;
  for (size_t e = (size_t)blockIdx.x * MVB + threadIdx.x; e < n; e += (size_t)gridDim.x * MVB)
    d[e] = fma(beta, d[e], s[e]);
}

// Right-hand sides of a group of map points: b[i * R + r] = S(map r,
// pixel i) with the table kernel (the reference's column, map minus pixel
// as lib/map_covar.cc:47-53), zero on padding rows and unused columns.
__global__ void k_mcolumns(KernelConsts kc, int n_pad, int R, int m,
                           const int* __restrict__ perm,
                           const double* __restrict__ px, const double* __restrict__ py,
                           const double* __restrict__ pz, const double* __restrict__ mp,
                           const double* __restrict__ table, double* __restrict__ b) {
  __shared__ double tf[TABLE_N];
  for (int k = threadIdx.x; k < TABLE_N; k += blockDim.x) tf[k] = table[k];
  __syncthreads();
  const size_t n = (size_t)n_pad * R;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / R), r = (int)(e % R);
    double v = 0.0;
    if (r < m && perm[i] >= 0)
      v = s_table_f64(mp[3 * r] - px[i], mp[3 * r + 1] - py[i], mp[3 * r + 2] - pz[i], kc, tf);
    b[e] = v;
  }
}

// sigma[r] = b_r . x_r for the converged right-hand sides (else 0): the map
// multiply of lib/map_covar.cc:100-110, S_mp[i, :] being the column b_r.
__global__ void __launch_bounds__(MVB) k_msigma(size_t n, const MState* st, const MShared* sh,
                                                const double* __restrict__ b,
                                                const double* __restrict__ x,
                                                unsigned int* counter, double* part,
                                                double* sigma) {
  __shared__ double tot[2 * MR_MAX];
  const int R = sh->R;
  double s = 0.0;
  for (size_t e = (size_t)blockIdx.x * MVB + threadIdx.x; e < n; e += (size_t)gridDim.x * MVB)
    s = fma(b[e], x[e], s);
  if (!grid_sum_by_rhs(R, s, 0.0, part, counter, tot)) return;
  for (int r = threadIdx.x; r < R; r += MVB) sigma[r] = st[r].converged ? tot[r] : 0.0;
}

}  // namespace

void map_covar_diag_multi(ds_operator* op, int n_map, const double* map_pts,
                          const ds_pcg_params& pp, double* sigma_m, int* iters, int* success) {
  cudaStream_t st = op->ctx->stream;
  require(pp.max_iter >= 0, "max_iter must be >= 0");
  require(pp.step_r > 0, "step_r must be > 0");
  // right-hand sides per solve: a power of two from 16 to 256 covering the
  // map points (or at least enough CTAs for the device)
  int R = MR;
  while (R < MR_MAX && R < n_map) R *= 2;
  const int np = op->pix.n_pad;
  const size_t nv = (size_t)np * R;
  const int g = mgrid(nv);
  const int hist_stride = std::max(pp.max_iter, 1) + 1;
  DevBuf<double> b, x, r, d, q, s, part, hist, mp, sig;
  DevBuf<MState> dst;
  DevBuf<MShared> dsh;
  b.alloc(nv);
  x.alloc(nv);
  r.alloc(nv);
  d.alloc(nv);
  q.alloc(nv);
  s.alloc(nv);
  part.alloc(std::max<size_t>((size_t)2 * R * g, (size_t)op->pix.n_tiles * R));
  hist.alloc((size_t)R * hist_stride);
  mp.alloc(3 * (size_t)R);
  sig.alloc(R);
  dst.alloc(R);
  dsh.alloc(1);
  ensure_op_pairs(op);
  MPairArgs pa{};
  pa.rx = op->pix.x.p;
  pa.ry = op->pix.y.p;
  pa.rz = op->pix.z.p;
  pa.row_ptr = op->pairs.row_ptr.p;
  pa.cols = op->pairs.cols.p;
  pa.row_order = op->pairs.row_order.p;
  pa.mask = op->pairs.mask.p;
  pa.wl = op->wl.p;
  pa.wr = op->wr.p;
  pa.e = op->e.p;
  pa.table = op->table.p;
  pa.part = part.p;
  pa.st = dst.p;
  pa.sh = dsh.p;
  MPairArgs prod = pa, resid = pa;
  prod.v = d.p;
  prod.out = q.p;
  prod.dotv = d.p;
  resid.v = x.p;
  resid.b = b.p;
  resid.out = r.p;
  const dim3 pgrid(op->pix.n_tiles, R / MR), pblock(TILE);

  std::vector<double> hp(3 * (size_t)R), hs(R);
  std::vector<MState> hst(R);
  MShared hsh{};
  hsh.max_iter = pp.max_iter;
  hsh.R = R;
  int h_done = 0;
  for (int g0 = 0; g0 < n_map; g0 += R) {
    const int m = std::min(R, n_map - g0);
    for (size_t k = 0; k < hp.size(); ++k)
      hp[k] = k < 3 * (size_t)m ? map_pts[3 * (size_t)g0 + k] : 0.0;
    DS_CUDA(cudaMemcpyAsync(mp.p, hp.data(), hp.size() * sizeof(double), cudaMemcpyHostToDevice,
                            st));
    DS_CUDA(cudaMemcpyAsync(dsh.p, &hsh, sizeof(hsh), cudaMemcpyHostToDevice, st));
    k_mcolumns<<<mgrid(nv), MVB, 0, st>>>(op->kc, np, R, m, op->pix.perm.p, op->pix.x.p,
                                          op->pix.y.p, op->pix.z.p, mp.p, op->table.p, b.p);
    DS_CHECK_LAUNCH();
    DS_CUDA(cudaMemsetAsync(x.p, 0, nv * sizeof(double), st));
    k_mnorm<<<g, MVB, 0, st>>>(nv, b.p, pp.tol, dst.p, dsh.p, part.p);
    DS_CHECK_LAUNCH();
    // r = b (x = 0), d = M^-1 r, delta, |r|  (lib/pcg.h:95-108)
    k_mupdate<3><<<g, MVB, 0, st>>>(nv, dst.p, dsh.p, x.p, r.p, d.p, q.p, s.p, b.p,
                                    op->pdiag.p, part.p, hist.p, hist_stride);
    DS_CHECK_LAUNCH();
    for (int it = 1; it < pp.max_iter; ++it) {
      k_mpair<false, true><<<pgrid, pblock, 0, st>>>(op->kc, prod);
      DS_CHECK_LAUNCH();
      if (it % pp.step_r == 0) {
        k_mupdate<1><<<g, MVB, 0, st>>>(nv, dst.p, dsh.p, x.p, r.p, d.p, q.p, s.p, b.p,
                                        op->pdiag.p, part.p, hist.p, hist_stride);
        DS_CHECK_LAUNCH();
        k_mpair<true, false><<<pgrid, pblock, 0, st>>>(op->kc, resid);
        DS_CHECK_LAUNCH();
        k_mupdate<2><<<g, MVB, 0, st>>>(nv, dst.p, dsh.p, x.p, r.p, d.p, q.p, s.p, b.p,
                                        op->pdiag.p, part.p, hist.p, hist_stride);
      } else {
        k_mupdate<0><<<g, MVB, 0, st>>>(nv, dst.p, dsh.p, x.p, r.p, d.p, q.p, s.p, b.p,
                                        op->pdiag.p, part.p, hist.p, hist_stride);
      }
      DS_CHECK_LAUNCH();
      k_mdir<<<g, MVB, 0, st>>>(nv, dst.p, dsh.p, s.p, d.p);
      DS_CHECK_LAUNCH();
      if (it % MCHECK == 0) {
        DS_CUDA(cudaMemcpyAsync(&h_done, &dsh.p->all_done, sizeof(int), cudaMemcpyDeviceToHost,
                                st));
        DS_CUDA(cudaStreamSynchronize(st));
        if (h_done) break;
      }
    }
    k_msigma<<<g, MVB, 0, st>>>(nv, dst.p, dsh.p, b.p, x.p, &dsh.p->counter[2], part.p, sig.p);
    DS_CHECK_LAUNCH();
    DS_CUDA(cudaMemcpyAsync(hs.data(), sig.p, R * sizeof(double), cudaMemcpyDeviceToHost, st));
    DS_CUDA(cudaMemcpyAsync(hst.data(), dst.p, R * sizeof(MState), cudaMemcpyDeviceToHost, st));
    DS_CUDA(cudaStreamSynchronize(st));
    for (int k = 0; k < m; ++k) {
      const MState& S = hst[k];
      int ok, its;
      if (!(S.norm_b > 0.0)) {  // lib/pcg.h:79-86
        puts("[WARNING] Requested PCG solve where |b| <= 0.0. Returning early.\n");
        ok = 0;
        its = 0;
      } else if (pp.max_iter <= 1) {  // lib/pcg.h:117-158 (as run_pcg)
        ok = pp.max_iter == 1 ? 0 : 1;
        its = 1;
      } else if (S.converged) {
        ok = 1;
        its = S.iter;
      } else {
        ok = 0;
        its = pp.max_iter;
      }
      if (!ok && S.norm_b > 0.0)
        puts("[WARNING] PCG reached max iteration before stop condition.");
      sigma_m[g0 + k] = ok ? hs[k] : 0.0;
      iters[g0 + k] = its;
      success[g0 + k] = ok;
    }
  }
}

}  // namespace ds
