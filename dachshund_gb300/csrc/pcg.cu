// Device-resident Jacobi-PCG (lib/pcg.h:27-160) and the BLAS-1 work around
// it (lib/linalg.cc:9-49), fused into three kernels per iteration:
//   K1  q = A d, with d.q reduced by the last CTA into alpha = delta / d.q
//   K2  x += alpha d;  r -= alpha q (or r = b - A x every step_r-th iteration);
//       s = M^-1 r;  r.s and r.r reduced by the last CTA, which also records
//       |r|, tests |r| <= tol |b| and raises the done flag
//   K3  d = s + beta d
// All scalars stay on the device.  Kernels of iterations enqueued after the
// solve converged see the done flag and return at once, so the host can run
// ahead of the device and read the flag only every few iterations.
// Reductions are deterministic (fixed tree order, no floating atomics).
#include <cmath>
#include <cstdio>

#include "ds_device.cuh"
#include "ds_ops.h"

namespace ds {

namespace {

constexpr int VB = 256;        // threads per vector-kernel CTA
constexpr int VGRID_MAX = 1024;

inline int vgrid(int n) { return std::max(1, std::min(VGRID_MAX, (n + VB - 1) / VB)); }

// Last CTA of K2 / init: fold r.s and r.r into the PCG state.
__device__ void pcg_finalize(PcgState* st, double rs, double rr, double* hist, double* dhist,
                             bool init) {
  if (init) {
    st->delta = rs;  // delta = r^T d, lib/pcg.h:104
    st->iter = 0;
    st->norm_r = sqrt(rr);
    hist[0] = st->norm_r;
    dhist[0] = rs;
    st->done = st->max_iter <= 1 ? 1 : 0;
    st->converged = 0;
    return;
  }
  st->delta_old = st->delta;
  st->delta = rs;                       // lib/pcg.h:58
  st->beta = st->delta / st->delta_old; // lib/pcg.h:61
  const int it = st->iter + 1;
  st->iter = it;
  st->norm_r = sqrt(rr);                // lib/pcg.h:123-126
  hist[it] = st->norm_r;
  dhist[it] = rs;
  if (st->norm_r <= st->tol_norm_b) {   // lib/pcg.h:130
    st->done = 1;
    st->converged = 1;
  } else if (it + 1 >= st->max_iter) {  // loop exit, lib/pcg.h:118,151
    st->done = 1;
    st->converged = 0;
  }
}

// mode 0: normal step (x, r recurrences + precondition + dots)
// mode 1: x update only (full-residual step, before the residual kernel)
// mode 2: precondition + dots only (full-residual step, after the residual)
// mode 3: initial d = M^-1 r + dots
template <int MODE>
__global__ void __launch_bounds__(VB) k_pcg_update(int n, PcgState* st, double* __restrict__ x,
                                                   double* __restrict__ r,
                                                   const double* __restrict__ d,
                                                   const double* __restrict__ q,
                                                   double* __restrict__ s,
                                                   const double* __restrict__ pdiag,
                                                   double* __restrict__ part, double* hist,
                                                   double* dhist) {
  if (MODE != 3 && st->done) return;
  __shared__ double red[VB / 32];
  const double alpha = (MODE == 0 || MODE == 1) ? st->alpha : 0.0;
  double rs = 0.0, rr = 0.0;
  for (int i = blockIdx.x * VB + threadIdx.x; i < n; i += gridDim.x * VB) {
    if (MODE == 0 || MODE == 1) x[i] = fma(alpha, d[i], x[i]);        // lib/pcg.h:39
    if (MODE == 1) continue;
    double ri = r[i];
    if (MODE == 0) {
      ri = fma(-alpha, q[i], ri);                                     // lib/pcg.h:48
      r[i] = ri;
    }
    const double si = ri / pdiag[i];                                  // lib/pcg.h:52
    s[i] = si;
    rs = fma(ri, si, rs);
    rr = fma(ri, ri, rr);
  }
  if (MODE == 1) return;
  const double brs = block_sum<VB>(rs, red);
  const double brr = block_sum<VB>(rr, red);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = brs;
    part[2 * blockIdx.x + 1] = brr;
  }
  if (last_block_arrive(&st->counter[1])) {
    const double trs = reduce_partials<VB>(part, gridDim.x, 2, 0, red);
    const double trr = reduce_partials<VB>(part, gridDim.x, 2, 1, red);
    if (threadIdx.x == 0) {
      pcg_finalize(st, trs, trr, hist, dhist, MODE == 3);
      st->counter[1] = 0;
    }
  }
}

// d = s + beta d (lib/pcg.h:62-64).
__global__ void __launch_bounds__(VB) k_pcg_direction(int n, const PcgState* st,
                                                      const double* __restrict__ s,
                                                      double* __restrict__ d) {
  if (st->done) return;
  const double beta = st->beta;
  for (int i = blockIdx.x * VB + threadIdx.x; i < n; i += gridDim.x * VB)
    d[i] = fma(beta, d[i], s[i]);
}

__global__ void k_gather(int n_pad, const int* __restrict__ perm, const double* __restrict__ src,
                         double* __restrict__ dst) {
  for (int i = blockIdx.x * VB + threadIdx.x; i < n_pad; i += gridDim.x * VB) {
    const int p = perm[i];
    dst[i] = p >= 0 ? src[p] : 0.0;
  }
}

__global__ void k_scatter(int n_pad, const int* __restrict__ perm, const double* __restrict__ src,
                          const double* __restrict__ scale, double* __restrict__ dst) {
  for (int i = blockIdx.x * VB + threadIdx.x; i < n_pad; i += gridDim.x * VB) {
    const int p = perm[i];
    if (p >= 0) dst[p] = scale ? src[i] * scale[i] : src[i];
  }
}

__global__ void k_mul(int n, const double* __restrict__ a, const double* __restrict__ b,
                      double* __restrict__ c) {
  for (int i = blockIdx.x * VB + threadIdx.x; i < n; i += gridDim.x * VB) c[i] = a[i] * b[i];
}

}  // namespace

void gather_sorted(const PointSet& ps, const double* src, double* dst, cudaStream_t st) {
  k_gather<<<vgrid(ps.n_pad), VB, 0, st>>>(ps.n_pad, ps.perm.p, src, dst);
  DS_CHECK_LAUNCH();
}

void scatter_sorted(const PointSet& ps, const double* src, const double* scale, double* dst,
                    cudaStream_t st) {
  k_scatter<<<vgrid(ps.n_pad), VB, 0, st>>>(ps.n_pad, ps.perm.p, src, scale, dst);
  DS_CHECK_LAUNCH();
}

void vec_mul(int n, const double* a, const double* b, double* c, cudaStream_t st) {
  k_mul<<<vgrid(n), VB, 0, st>>>(n, a, b, c);
  DS_CHECK_LAUNCH();
}

void ensure_op_pairs(ds_operator* op) {
  if (op->pairs_built) return;
  build_pair_list(op->pairs, op->pix, op->pix, op->kc, op->ctx->stream);
  op->pairs_built = true;
}

PairArgs op_pair_args(ds_operator* op, const double* v, double* out) {
  ensure_op_pairs(op);
  PairArgs a{};
  a.rx = a.cx = op->pix.x.p;
  a.ry = a.cy = op->pix.y.p;
  a.rz = a.cz = op->pix.z.p;
  a.row_ptr = op->pairs.row_ptr.p;
  a.cols = op->pairs.cols.p;
  a.mask = op->pairs.mask.p;
  a.row_order = op->pairs.row_order.p;
  a.n_row_tiles = op->pix.n_tiles;
  a.wl = op->wl.p;
  a.wr = op->wr.p;
  a.e = op->e.p;
  a.b = op->b.p;
  a.v = v;
  a.vrow = v;
  a.out = out;
  a.table = op->table.p;
  a.n_tile_pairs = op->pairs.n_pairs;
  a.prof = &op->ctx->prof;
  return a;
}

void op_apply_sorted(ds_operator* op, int epi, const double* v, double* out, cudaStream_t st) {
  if (op->use_dense) {
    dense_apply(op, epi == EPI_RESIDUAL, v, out, nullptr, nullptr, nullptr, st);
    return;
  }
  PairArgs a = op_pair_args(op, v, out);
  launch_pair_f64(op->kc, epi, a, st);
}

void ensure_pcg_workspace(ds_operator* op) {
  const size_t np = op->pix.n_pad;
  op->x.alloc(np);
  op->r.alloc(np);
  op->d.alloc(np);
  op->q.alloc(np);
  op->s.alloc(np);
  op->partial.alloc(std::max<size_t>(2 * VGRID_MAX, op->pix.n_tiles));
  // + 2 n_pad: the per-skewer (r.z, |r|^2) partials of the preconditioned
  // mixed form, after the n_tiles p.q partials
  op->partial2.alloc(std::max((size_t)2 * VGRID_MAX, (size_t)op->pix.n_tiles) +
                     2 * (size_t)op->pix.n_pad);
  op->state.alloc(1);
  op->h_flag.alloc(64);
}

// Runs Jacobi-PCG on op with x (sorted, padded, device) as the initial guess.
void run_pcg(ds_operator* op, const ds_pcg_params& pp, ds_pcg_result& res, double* hist_out) {
  cudaStream_t st = op->ctx->stream;
  const int np = op->pix.n_pad;
  require(pp.max_iter >= 0, "max_iter must be >= 0");
  require(pp.step_r > 0, "step_r must be > 0");
  op->hist.alloc((size_t)std::max(pp.max_iter, 1) + 1);
  op->dhist.alloc((size_t)std::max(pp.max_iter, 1) + 1);

  PcgState h{};
  h.max_iter = pp.max_iter;
  h.norm_b = op->norm_b;
  h.tol_norm_b = pp.tol * op->norm_b;  // lib/pcg.h:93
  DS_CUDA(cudaMemcpyAsync(op->state.p, &h, sizeof(h), cudaMemcpyHostToDevice, st));

  cudaEvent_t ev0, ev1;
  DS_CUDA(cudaEventCreate(&ev0));
  DS_CUDA(cudaEventCreate(&ev1));
  DS_CUDA(cudaEventRecord(ev0, st));

  PcgState* S = op->state.p;
  const int g = vgrid(np);
  // r = b - A x; d = M^-1 r; delta = r.d; |r|  (lib/pcg.h:95-108)
  op_apply_sorted(op, EPI_RESIDUAL, op->x.p, op->r.p, st);
  k_pcg_update<3><<<g, VB, 0, st>>>(np, S, op->x.p, op->r.p, op->q.p, op->q.p, op->d.p,
                                    op->pdiag.p, op->partial.p, op->hist.p, op->dhist.p);
  DS_CHECK_LAUNCH();

  PairArgs prod = op_pair_args(op, op->d.p, op->q.p);
  prod.dotv = op->d.p;
  prod.dot_partial = op->partial2.p;
  prod.pcg = S;
  prod.counter = &S->counter[0];
  prod.skip_flag = &S->done;
  PairArgs resid = op_pair_args(op, op->x.p, op->r.p);
  resid.skip_flag = &S->done;

  constexpr int CHECK = 8;     // read the done flag every CHECK iterations
  constexpr int NSLOT = 64;
  cudaEvent_t evs[NSLOT];
  for (auto& e : evs) DS_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  int issued = 0, waited = 0;
  for (int it = 1; it < pp.max_iter; ++it) {
    if (op->use_dense)  // q = A d, alpha
      dense_apply(op, false, op->d.p, op->q.p, op->d.p, S, &S->done, st);
    else
      launch_pair_f64(op->kc, EPI_PRODUCT, prod, st);
    if (it % pp.step_r == 0) {
      k_pcg_update<1><<<g, VB, 0, st>>>(np, S, op->x.p, op->r.p, op->d.p, op->q.p, op->s.p,
                                        op->pdiag.p, op->partial.p, op->hist.p, op->dhist.p);
      DS_CHECK_LAUNCH();
      if (op->use_dense)  // r = b - A x
        dense_apply(op, true, op->x.p, op->r.p, nullptr, nullptr, &S->done, st);
      else
        launch_pair_f64(op->kc, EPI_RESIDUAL, resid, st);
      k_pcg_update<2><<<g, VB, 0, st>>>(np, S, op->x.p, op->r.p, op->d.p, op->q.p, op->s.p,
                                        op->pdiag.p, op->partial.p, op->hist.p, op->dhist.p);
    } else {
      k_pcg_update<0><<<g, VB, 0, st>>>(np, S, op->x.p, op->r.p, op->d.p, op->q.p, op->s.p,
                                        op->pdiag.p, op->partial.p, op->hist.p, op->dhist.p);
    }
    DS_CHECK_LAUNCH();
    k_pcg_direction<<<g, VB, 0, st>>>(np, S, op->s.p, op->d.p);
    DS_CHECK_LAUNCH();
    if (it % CHECK == 0) {
      const int slot = issued % NSLOT;
      DS_CUDA(cudaMemcpyAsync(&op->h_flag.p[slot], &S->done, sizeof(int),
                              cudaMemcpyDeviceToHost, st));
      DS_CUDA(cudaEventRecord(evs[slot], st));
      ++issued;
      // Stay at most two checks ahead of the device.
      if (issued - waited > 2) {
        const int ws = waited % NSLOT;
        DS_CUDA(cudaEventSynchronize(evs[ws]));
        ++waited;
        if (op->h_flag.p[ws]) break;
      }
    }
  }
  DS_CUDA(cudaEventRecord(ev1, st));
  DS_CUDA(cudaMemcpyAsync(&h, S, sizeof(h), cudaMemcpyDeviceToHost, st));
  DS_CUDA(cudaStreamSynchronize(st));
  float ms = 0.f;
  DS_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
  for (auto& e : evs) cudaEventDestroy(e);
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);

  const int n_hist = h.iter + 1;
  std::vector<double> hh(n_hist), dh(n_hist);
  DS_CUDA(cudaMemcpyAsync(hh.data(), op->hist.p, n_hist * sizeof(double), cudaMemcpyDeviceToHost, op->ctx->stream));
  DS_CUDA(cudaStreamSynchronize(op->ctx->stream));
  DS_CUDA(cudaMemcpyAsync(dh.data(), op->dhist.p, n_hist * sizeof(double), cudaMemcpyDeviceToHost, op->ctx->stream));
  DS_CUDA(cudaStreamSynchronize(op->ctx->stream));
  if (hist_out)
    for (int k = 0; k < n_hist; ++k) hist_out[k] = hh[k];

  res.norm_b = op->norm_b;
  res.final_norm = h.norm_r;
  res.seconds = ms * 1e-3;
  res.n_outer = 0;
  res.n_inner = h.iter;
  // lib/pcg.h:117-158: the loop variable leaves the loop at 1 when
  // max_iter <= 1, and success is false only when it equals max_iter, so
  // max_iter = 1 fails and max_iter = 0 succeeds, both with one iteration.
  if (pp.max_iter <= 1) {
    res.success = pp.max_iter == 1 ? 0 : 1;
    res.num_iters = 1;
  } else if (h.converged) {
    res.success = 1;
    res.num_iters = h.iter;
  } else {
    res.success = 0;
    res.num_iters = pp.max_iter;
  }
  if (pp.verbose) {
    // The reference's trace (lib/pcg.h:112-141, 151-155).
    printf("[PCG] Solving %i x %i problem.\n", op->n, op->n);
    printf("    Goal |r| < (tol) |b| = %e,  delta = %e\n", h.tol_norm_b, dh[0]);
    for (int k = 1; k < n_hist; ++k) {
      if (hh[k] <= h.tol_norm_b)
        printf("    iter %i reached |r| = %e < tol |b| = %e\n", k, hh[k], h.tol_norm_b);
      else
        printf("    iter %i, |r| %e, delta %e\n", k, hh[k], dh[k]);
    }
  }
  // printed on every failed solve, as lib/pcg.h:151-155 does
  if (!res.success) puts("[WARNING] PCG reached max iteration before stop condition.");
}

}  // namespace ds
