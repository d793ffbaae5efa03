// Mixed-precision Jacobi-PCG: FP32 Krylov iteration with FP64 reliable
// updates (residual replacement, in the manner of Sleijpen & van der Vorst).
//
//   FP64: the iterate x (x += alpha p every iteration: one FP64 FMA per
//         pixel), the right-hand side b, the true residual r64 = b - A x
//         (FP64-accurate matrix-free kernel, same operator as the plain
//         form), every CG scalar (r.z, p.q, |r| are FP32 vectors summed in
//         FP64), and the stopping test |r64| <= tol |b|.
//   FP32: the search direction p, q = A32 p (FP32 MUFU kernel), the residual
//         recurrence r and z = M^-1 r.
// A reliable update recomputes r64 from x and restarts the recurrence from
// float(r64) while keeping the search direction.  It fires when the
// recurrence residual has dropped by `delta` since the last update, when it
// reaches tol |b|, at the iteration cap, or when the recurrence stagnates
// (then the direction is dropped, beta = 0); the solve ends only on an FP64
// residual.  Per iteration: K1 q = A32 p (+ p.q, alpha), K2 x and the
// recurrences, K5 / K6 the update (they return at once on a device flag
// unless one is due), K7 the new direction.
#include <algorithm>
#include <cmath>
#include <cstdio>

#include "ds_device.cuh"
#include "ds_f32.h"
#include "ds_learned.h"
#include "ds_skewer.h"
#include "ds_mixed_dev.cuh"
#include "ds_ops.h"

namespace ds {

void OpF32Deleter::operator()(OpF32* p) const { delete p; }
void MapF32Deleter::operator()(MapF32* p) const { delete p; }

namespace {

constexpr int VB = 256;
// Grid cap of the vector kernels (grid-stride loops): 2 CTAs per SM keeps the
// last CTA's reduction over the partials short (measured: 304 CTAs beat 1024
// by ~5 us per iteration on 262,144 pixels).
constexpr int VGRID_MAX = 304;
inline int vgrid(int n) { return std::max(1, std::min(VGRID_MAX, (n + VB - 1) / VB)); }

const double LOG2E = 1.4426950408889634;

// ---- FP32 point preparation ----------------------------------------------

__global__ void k_f32_origins(int n_tiles, const double* __restrict__ box, double sx, double sy,
                              double sz, float4* __restrict__ orig) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tiles) return;
  const double* b = box + (size_t)t * 6;
  orig[t] = make_float4((float)(0.5 * (b[0] + b[3]) * sx), (float)(0.5 * (b[1] + b[4]) * sy),
                        (float)(0.5 * (b[2] + b[5]) * sz), 0.f);
}

__global__ void k_f32_xi(int n_pad, const double* __restrict__ x, const double* __restrict__ y,
                         const double* __restrict__ z, double sx, double sy, double sz,
                         const float4* __restrict__ orig, float4* __restrict__ xi,
                         float* __restrict__ blockmax) {
  __shared__ float sm[VB];
  const int i = blockIdx.x * VB + threadIdx.x;
  float a = 0.f;
  if (i < n_pad) {
    const float4 o = orig[i / TILE];
    const float fx = (float)(x[i] * sx - (double)o.x);
    const float fy = (float)(y[i] * sy - (double)o.y);
    const float fz = (float)(z[i] * sz - (double)o.z);
    a = fmaf(fx, fx, fmaf(fy, fy, fz * fz));
    xi[i] = make_float4(fx, fy, fz, a);
  }
  sm[threadIdx.x] = a;
  __syncthreads();
  for (int s = VB / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sm[threadIdx.x] = fmaxf(sm[threadIdx.x], sm[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) blockmax[blockIdx.x] = sm[0];
}

// Row / column coefficients of the FP32 operator from the FP64 ones.
__global__ void k_f32_coeffs(int n_pad, int expanded, double var_s, const float4* __restrict__ xi,
                             const double* __restrict__ wl, const double* __restrict__ wr,
                             const double* __restrict__ e, const double* __restrict__ pdiag,
                             float* __restrict__ rowf, float* __restrict__ colw,
                             float* __restrict__ ediag, float* __restrict__ pd) {
  for (int i = blockIdx.x * VB + threadIdx.x; i < n_pad; i += gridDim.x * VB) {
    const double scale = expanded ? exp2(-(double)xi[i].w) : 1.0;
    rowf[i] = (float)(wl[i] * var_s * scale);
    colw[i] = (float)wr[i];
    ediag[i] = (float)e[i];
    pd[i] = (float)pdiag[i];
  }
}

__global__ void k_fill_f32(int n, float v, float* __restrict__ out) {
  for (int i = blockIdx.x * VB + threadIdx.x; i < n; i += gridDim.x * VB) out[i] = v;
}

__global__ void k_d2f(int n, const double* __restrict__ in, float* __restrict__ out) {
  for (int i = blockIdx.x * VB + threadIdx.x; i < n; i += gridDim.x * VB) out[i] = (float)in[i];
}

// ---- the iteration kernels -----------------------------------------------

// Zero test of the initial guess: flag = 1 when every entry is 0.
__global__ void k_is_zero(int n, const double* __restrict__ x, int* __restrict__ flag) {
  for (int i = blockIdx.x * VB + threadIdx.x; i < n; i += gridDim.x * VB)
    if (x[i] != 0.0) *flag = 0;
}

// x32 = float(x0) for the FP32 initial residual (skipped when x0 == 0).
__global__ void k_x_to_f32(int n, const int* x_zero, const double* __restrict__ x,
                           float* __restrict__ x32) {
  if (*x_zero) return;
  for (int i = blockIdx.x * VB + threadIdx.x; i < n; i += gridDim.x * VB) x32[i] = (float)x[i];
}

// r64 = b - q32 with q32 = A32 x0 (the FP32 product), and the decision on
// the FP64-accurate initial residual: it is needed only when x0 != 0 and
// |b - A32 x0| <= 1e-5 |b| (the FP32 operator's error, ~1e-6 |b|, could then
// decide convergence); otherwise the first reliable update replaces the
// FP32 residual.
__global__ void __launch_bounds__(VB) k_r32_init(int n, MixedState* st, const int* x_zero,
                                                 const double* __restrict__ b,
                                                 const float* __restrict__ q32,
                                                 double* __restrict__ r64,
                                                 double* __restrict__ part) {
  __shared__ double red[VB / 32];
  const bool zero = *x_zero != 0;
  double rr = 0.0;
  if (!zero)
    for (int i = blockIdx.x * VB + threadIdx.x; i < n; i += gridDim.x * VB) {
      const double ri = b[i] - (double)q32[i];
      r64[i] = ri;
      rr = fma(ri, ri, rr);
    }
  const double brr = block_sum<VB>(rr, red);
  if (threadIdx.x == 0) part[blockIdx.x] = brr;
  if (last_block_arrive(&st->counter[1])) {
    const double trr = reduce_partials<VB>(part, gridDim.x, 1, 0, red);
    if (threadIdx.x == 0) {
      st->init_skip = (zero || sqrt(trr) > 1e-5 * st->norm_b) ? 1 : 0;
      st->counter[1] = 0;
    }
  }
}

// r = float(r64) (or b when x0 == 0); z = r / pd; p = z; r.z, |r|.
__global__ void __launch_bounds__(VB) k_mx_init(int n, MixedState* st, const int* x_zero,
                                                const double* __restrict__ b,
                                                const double* __restrict__ r64,
                                                float* __restrict__ r, float* __restrict__ z,
                                                float* __restrict__ p,
                                                const float* __restrict__ pd,
                                                double* __restrict__ part, double* hist,
                                                double* htrue) {
  __shared__ double red[VB / 32];
  const bool zero = *x_zero != 0;
  double rz = 0.0, rr = 0.0;
  for (int i = blockIdx.x * VB + threadIdx.x; i < n; i += gridDim.x * VB) {
    const double rd = zero ? b[i] : r64[i];
    const float ri = (float)rd;
    const float zi = ri / pd[i];
    r[i] = ri;
    z[i] = zi;
    p[i] = zi;
    rz = fma((double)ri, (double)zi, rz);
    rr = fma(rd, rd, rr);
  }
  const double brz = block_sum<VB>(rz, red);
  const double brr = block_sum<VB>(rr, red);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = brz;
    part[2 * blockIdx.x + 1] = brr;
  }
  if (last_block_arrive(&st->counter[1])) {
    const double trz = reduce_partials<VB>(part, gridDim.x, 2, 0, red);
    const double trr = reduce_partials<VB>(part, gridDim.x, 2, 1, red);
    if (threadIdx.x == 0) {
      st->rz = trz;
      st->rnorm = st->rtrue = st->rmax = st->rbest = sqrt(trr);
      st->it_best = 0;
      st->stalled = 0;
      st->iter = 0;
      st->n_updates = 0;
      st->need_update = 0;
      st->skip_update = 1;
      hist[0] = st->rtrue;
      htrue[0] = st->rtrue;
      st->converged = st->rtrue <= st->tol_norm_b ? 1 : 0;
      st->done = (st->converged || st->max_iter <= 0) ? 1 : 0;
      st->counter[1] = 0;
    }
  }
}

// K2: x += alpha p (FP64); r -= alpha q; z = r / pd; r.z, |r|; decide on an
// update.
__global__ void __launch_bounds__(VB) k_mx_update(int n, MixedState* st, double* __restrict__ x,
                                                  float* __restrict__ r, float* __restrict__ z,
                                                  const float* __restrict__ p,
                                                  const float* __restrict__ q,
                                                  const float* __restrict__ pd,
                                                  double* __restrict__ part, double* hist) {
  if (st->done) return;
  __shared__ double red[VB / 32];
  const double alpha_d = st->alpha;
  const float alpha = (float)alpha_d;
  double rz = 0.0, rr = 0.0;
  for (int i = blockIdx.x * VB + threadIdx.x; i < n; i += gridDim.x * VB) {
    x[i] = fma(alpha_d, (double)p[i], x[i]);
    const float ri = fmaf(-alpha, q[i], r[i]);
    const float zi = ri / pd[i];
    r[i] = ri;
    z[i] = zi;
    rz = fma((double)ri, (double)zi, rz);
    rr = fma((double)ri, (double)ri, rr);
  }
  const double brz = block_sum<VB>(rz, red);
  const double brr = block_sum<VB>(rr, red);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = brz;
    part[2 * blockIdx.x + 1] = brr;
  }
  if (last_block_arrive(&st->counter[1])) {
    const double trz = reduce_partials<VB>(part, gridDim.x, 2, 0, red);
    const double trr = reduce_partials<VB>(part, gridDim.x, 2, 1, red);
    if (threadIdx.x == 0) {
      st->rz_old = st->rz;
      st->rz = trz;
      st->rnorm = sqrt(trr);
      const int it = st->iter + 1;
      st->iter = it;
      hist[it] = st->rnorm;
      st->rmax = fmax(st->rmax, st->rnorm);
      const bool upd = update_due(st, it);
      st->need_update = upd ? 1 : 0;
      st->skip_update = upd ? 0 : 1;
      st->beta = st->rz / st->rz_old;
      st->counter[1] = 0;
    }
  }
}

// K6: r = float(r64); z = r / pd; r.z and |r64| (FP64); stop or continue.
__global__ void __launch_bounds__(VB) k_mx_replace(int n, MixedState* st,
                                                   const double* __restrict__ r64,
                                                   float* __restrict__ r, float* __restrict__ z,
                                                   const float* __restrict__ pd,
                                                   double* __restrict__ part, double* hist,
                                                   double* htrue) {
  if (st->done || !st->need_update) return;
  __shared__ double red[VB / 32];
  double rz = 0.0, rr = 0.0;
  for (int i = blockIdx.x * VB + threadIdx.x; i < n; i += gridDim.x * VB) {
    const double rd = r64[i];
    const float ri = (float)rd;
    const float zi = ri / pd[i];
    r[i] = ri;
    z[i] = zi;
    rz = fma((double)ri, (double)zi, rz);
    rr = fma(rd, rd, rr);
  }
  const double brz = block_sum<VB>(rz, red);
  const double brr = block_sum<VB>(rr, red);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = brz;
    part[2 * blockIdx.x + 1] = brr;
  }
  if (last_block_arrive(&st->counter[1])) {
    const double trz = reduce_partials<VB>(part, gridDim.x, 2, 0, red);
    const double trr = reduce_partials<VB>(part, gridDim.x, 2, 1, red);
    if (threadIdx.x == 0) {
      const double rt = sqrt(trr);
      st->rtrue = rt;
      htrue[++st->n_updates] = rt;
      hist[st->iter] = rt;
      if (rt <= st->tol_norm_b) {
        st->done = 1;
        st->converged = 1;
      } else if (st->iter >= st->max_iter) {
        st->done = 1;
      } else {
        st->rz = trz;  // rz_old keeps the previous iteration's r.z
        restart_after_update(st, rt, trz);
      }
      // the update is done: no FP64 residual until K2 asks for one again
      // (every block read the flags before it arrived)
      st->need_update = 0;
      st->skip_update = 1;
      st->counter[1] = 0;
    }
  }
}

// K7: p = z + beta p (beta from K2, or from K6's restart after an update);
// after an update the last block clears the update flags.  Every block reads
// the flag before it arrives, and the flag is cleared only after all have
// arrived.
__global__ void __launch_bounds__(VB) k_mx_dir(int n, MixedState* st,
                                               const float* __restrict__ z,
                                               float* __restrict__ p) {
  const bool upd = st->need_update != 0;
  if (!st->done) {
    const float beta = (float)st->beta;
    for (int i = blockIdx.x * VB + threadIdx.x; i < n; i += gridDim.x * VB)
      p[i] = fmaf(beta, p[i], z[i]);
  }
  if (upd && last_block_arrive(&st->counter[2]) && threadIdx.x == 0) {
    st->need_update = 0;
    st->skip_update = 1;
    st->counter[2] = 0;
  }
}

// ---- band preconditioner (M^-1 = L L^T) ---------------------------------------
// The same reliable-update iteration with z = M^-1 r for a band factor L in
// slot order (a skewer per block of slots, or a cluster of neighbouring
// skewers in z order; L has no entries between blocks, padding slots have
// r = 0).  One thread per slot, PCB slots per CTA plus `band` halo slots on
// each side: the CTA forms its slots' r (updated in MODE 0), t = L^T r on
// its slots and the `band` before them, and z = L t on its own slots, writes
// its (r.z, |r|^2) partials, and the last CTA to finish does the scalar
// bookkeeping of K2 (MODE 0), K6 (MODE 1) or the start (MODE 2).  Slot ->
// record (crec, or the slot itself) -> vector index (inv, or the record
// itself in record order).
constexpr int PCB = 256;       // slots per CTA
constexpr int PC_MAX_BAND = 32;

struct PcArgs {
  int n_slots, band;
  MixedState* st;
  const int* x_zero;
  const int* crec;  // slot -> record (null: the slot itself)
  const int* inv;   // record -> vector index (null: the record itself)
  const float* L;   // band + 1 planes of n_slots
  double* x;
  const float* rin;  // MODE 0: r of the previous iteration
  float* rout;       // r of this iteration
  float* z;
  float* p;
  const float* q;
  const double* b;
  const double* r64;
  double* part;
  double* hist;
  double* htrue;
};

// BAND >= 0: the band as a constant (loops unrolled, all L loads of a slot
// in flight together); -1: a.band at run time.
template <int MODE, int BAND>
__global__ void __launch_bounds__(PCB) k_pc_iter(PcArgs a) {
  MixedState* st = a.st;
  const int n_slots = a.n_slots;
  const int band = BAND >= 0 ? BAND : a.band;
  const int* __restrict__ crec = a.crec;
  const int* __restrict__ inv = a.inv;
  const float* __restrict__ L = a.L;
  double* __restrict__ x = a.x;
  const float* __restrict__ rin = a.rin;
  float* __restrict__ rout = a.rout;
  float* __restrict__ z = a.z;
  float* __restrict__ p = a.p;
  const float* __restrict__ q = a.q;
  const double* __restrict__ b = a.b;
  const double* __restrict__ r64 = a.r64;
  double* __restrict__ part = a.part;
  double* hist = a.hist;
  double* htrue = a.htrue;
  const int* x_zero = a.x_zero;
  if (MODE == 0 && st->done) return;
  if (MODE == 1 && (st->done || !st->need_update)) return;
  __shared__ float rs[PCB + 2 * PC_MAX_BAND];  // r of slots s0 - band ..
  __shared__ float ts[PCB + PC_MAX_BAND];      // t of slots s0 - band ..
  __shared__ double red[PCB / 32];
  const int tid = threadIdx.x;
  const int s0 = blockIdx.x * PCB;
  const size_t ns = (size_t)n_slots;
  auto index_of = [&](int slot) -> int {
    if (slot < 0 || slot >= n_slots) return -1;
    const int rec = crec ? crec[slot] : slot;
    return rec < 0 ? -1 : inv ? inv[rec] : rec;
  };
  const double alpha_d = MODE == 0 ? st->alpha : 0.0;
  const bool from_b = MODE == 2 && *x_zero;
  // r of the CTA's slots and halos: MODE 0 updates the previous r (rin, not
  // written by this kernel, so halos read the same values as their owners)
  for (int i = tid; i < PCB + 2 * band; i += PCB) {
    const int pos = index_of(s0 - band + i);
    float v = 0.f;
    if (pos >= 0)
      v = MODE == 0 ? fmaf(-(float)alpha_d, q[pos], rin[pos])
                    : (float)(from_b ? b[pos] : r64[pos]);
    rs[i] = v;
  }
  __syncthreads();
  const int k = s0 + tid;  // this thread's slot
  const int own = index_of(k);
  const float ri = rs[tid + band];
  double rd = 0.0;
  if (own >= 0) {
    rout[own] = ri;
    if (MODE == 0) {
      x[own] = fma(alpha_d, (double)p[own], x[own]);
      rd = ri;
    } else {
      rd = from_b ? b[own] : r64[own];
    }
  }
  for (int i = tid; i < PCB + band; i += PCB) {  // t of slot s0 - band + i
    const int j = s0 - band + i;
    float t = 0.f;
    if (j >= 0) {
#pragma unroll
      for (int m = 0; m <= (BAND >= 0 ? BAND : PC_MAX_BAND); ++m)
        if (m <= band && j + m < n_slots) t = fmaf(L[(size_t)m * ns + j + m], rs[i + m], t);
    }
    ts[i] = t;
  }
  __syncthreads();
  float zk = 0.f;
  if (k < n_slots) {
#pragma unroll
    for (int m = 0; m <= (BAND >= 0 ? BAND : PC_MAX_BAND); ++m)
      if (m <= band) zk = fmaf(L[(size_t)m * ns + k], ts[tid + band - m], zk);
  }
  if (own >= 0) {
    z[own] = zk;
    if (MODE == 2) p[own] = zk;
  }
  const double srz = block_sum<PCB>(own >= 0 ? (double)ri * (double)zk : 0.0, red);
  const double srr = block_sum<PCB>(rd * rd, red);
  if (tid == 0) {
    part[2 * blockIdx.x] = srz;
    part[2 * blockIdx.x + 1] = srr;
  }
  if (!last_block_arrive(&st->counter[3])) return;
  const double trz = reduce_partials<PCB>(part, gridDim.x, 2, 0, red);
  const double trr = reduce_partials<PCB>(part, gridDim.x, 2, 1, red);
  if (tid != 0) return;
  st->counter[3] = 0;
  if (MODE == 2) {
    st->rz = trz;
    st->rnorm = st->rtrue = st->rmax = st->rbest = sqrt(trr);
    st->it_best = 0;
    st->stalled = 0;
    st->iter = 0;
    st->n_updates = 0;
    st->need_update = 0;
    st->skip_update = 1;
    hist[0] = st->rtrue;
    htrue[0] = st->rtrue;
    st->converged = st->rtrue <= st->tol_norm_b ? 1 : 0;
    st->done = (st->converged || st->max_iter <= 0) ? 1 : 0;
  } else if (MODE == 0) {
    st->rz_old = st->rz;
    st->rz = trz;
    st->rnorm = sqrt(trr);
    const int it = st->iter + 1;
    st->iter = it;
    hist[it] = st->rnorm;
    st->rmax = fmax(st->rmax, st->rnorm);
    const bool upd = update_due(st, it);
    st->need_update = upd ? 1 : 0;
    st->skip_update = upd ? 0 : 1;
    st->beta = st->rz / st->rz_old;
  } else {
    const double rt = sqrt(trr);
    st->rtrue = rt;
    htrue[++st->n_updates] = rt;
    hist[st->iter] = rt;
    if (rt <= st->tol_norm_b) {
      st->done = 1;
      st->converged = 1;
    } else if (st->iter >= st->max_iter) {
      st->done = 1;
    } else {
      st->rz = trz;
      restart_after_update(st, rt, trz);
    }
    st->need_update = 0;  // as k_mx_replace: the update is done
    st->skip_update = 1;
  }
}

template <int MODE>
void pc_iter(const PcArgs& a, cudaStream_t st) {
  const unsigned grid = (unsigned)((a.n_slots + PCB - 1) / PCB);
  if (a.band == 16)
    k_pc_iter<MODE, 16><<<grid, PCB, 0, st>>>(a);
  else if (a.band == 2)
    k_pc_iter<MODE, 2><<<grid, PCB, 0, st>>>(a);
  else
    k_pc_iter<MODE, -1><<<grid, PCB, 0, st>>>(a);
  DS_CHECK_LAUNCH();
}

}  // namespace

void build_f32_points(F32Points& fp, const PointSet& ps, double sx, double sy, double sz,
                      cudaStream_t st) {
  fp.orig.alloc(ps.n_tiles);
  fp.xi.alloc(ps.n_pad);
  k_f32_origins<<<(ps.n_tiles + 127) / 128, 128, 0, st>>>(ps.n_tiles, ps.box.p, sx, sy, sz,
                                                          fp.orig.p);
  DS_CHECK_LAUNCH();
  const int nb = (ps.n_pad + VB - 1) / VB;
  DevBuf<float> bm;
  bm.alloc(nb);
  k_f32_xi<<<nb, VB, 0, st>>>(ps.n_pad, ps.x.p, ps.y.p, ps.z.p, sx, sy, sz, fp.orig.p, fp.xi.p,
                              bm.p);
  DS_CHECK_LAUNCH();
  std::vector<float> h(nb);
  DS_CUDA(cudaMemcpyAsync(h.data(), bm.p, nb * sizeof(float), cudaMemcpyDeviceToHost, st));
  DS_CUDA(cudaStreamSynchronize(st));
  fp.max_a = *std::max_element(h.begin(), h.end());
}

// Scales of the exact kernel in log2 units: |dX|^2 = arg * log2(e).
static void exact_scales(const KernelConsts& kc, double& sp, double& sq) {
  sp = std::sqrt(kc.c_perp * LOG2E);
  sq = std::sqrt(kc.c_para * LOG2E);
}

void ensure_op_f32(ds_operator* op, double inner_cut) {
  if (op->f32 && op->f32->inner_cut == inner_cut) return;
  require(op->kc.eval == DS_EVAL_EXACT,
          "the mixed-precision form evaluates the exact kernel (eval = DS_EVAL_EXACT)");
  cudaStream_t st = op->ctx->stream;
  std::unique_ptr<OpF32, OpF32Deleter> f(new OpF32());
  f->inner_cut = inner_cut;
  double sp, sq;
  exact_scales(op->kc, sp, sq);
  build_f32_points(f->pts, op->pix, sp, sp, sq, st);
  // 2^|xi|^2 must stay well inside FP32 range for the EXPANDED formula.
  f->formula = f->pts.max_a <= 60.0 ? F32_EXPANDED : F32_DIRECT;
  const int np = op->pix.n_pad;
  f->rowf.alloc(np);
  f->colw.alloc(np);
  f->ediag.alloc(np);
  f->pdiag.alloc(np);
  k_f32_coeffs<<<vgrid(np), VB, 0, st>>>(np, f->formula == F32_EXPANDED, op->kc.var_s,
                                         f->pts.xi.p, op->wl.p, op->wr.p, op->e.p, op->pdiag.p,
                                         f->rowf.p, f->colw.p, f->ediag.p, f->pdiag.p);
  DS_CHECK_LAUNCH();
  f->p.alloc(np);
  f->q.alloc(np);
  f->r.alloc(np);
  f->z.alloc(np);
  f->state.alloc(1);
  f->use_ff = ff_usable(op->kc);
  if (f->use_ff) build_ff_points(f->ffd, op->pix, op->kc, st);
  DS_CUDA(cudaStreamSynchronize(st));
  op->f32 = std::move(f);
}

// The FP32 pair kernels' tile-pair list at the inner cutoff, built on the
// first solve that runs them (the structured inner product needs none).
void ensure_f32_pairs(ds_operator* op) {
  OpF32& f = *op->f32;
  if (f.pairs_built) return;
  KernelConsts kc = op->kc;
  kc.cull_arg = f.inner_cut * (1.0 + 1e-9);
  build_pair_list(f.pairs, op->pix, op->pix, kc, op->ctx->stream);
  build_slice_items(f.pairs, op->ctx->stream);
  f.pairs_built = true;
}

F32Args op_f32_args(ds_operator* op, const float* v, float* out) {
  OpF32& f = *op->f32;
  F32Args a{};
  a.rxi = a.cxi = f.pts.xi.p;
  a.rorig = a.corig = f.pts.orig.p;
  a.row_ptr = f.pairs.row_ptr.p;
  a.cols = f.pairs.cols.p;
  a.mask = f.pairs.mask.p;
  a.item_ptr = f.pairs.item_ptr.p;
  a.items = f.pairs.items.p;
  a.row_order = f.pairs.row_order.p;
  a.n_row_tiles = op->pix.n_tiles;
  a.colw = f.colw.p;
  a.v = v;
  a.rowf = f.rowf.p;
  a.ediag = f.ediag.p;
  a.vrow = v;
  a.out = out;
  a.n_tile_pairs = f.pairs.n_pairs;
  a.prof = &op->ctx->prof;
  return a;
}

void run_mixed(ds_operator* op, const ds_mixed_params& mp, ds_pcg_result& res,
               double* hist_out) {
  cudaStream_t st = op->ctx->stream;
  ensure_pcg_workspace(op);
  const double inner_cut = mp.inner_cutoff > 0.0 ? mp.inner_cutoff : DS_DEFAULT_INNER_CUTOFF;
  ensure_op_f32(op, inner_cut);
  OpF32& f = *op->f32;
  const int np = op->pix.n_pad;
  const int max_iter = std::max(mp.max_iter, 0);
  f.hist.alloc((size_t)max_iter + 2);
  f.htrue.alloc((size_t)max_iter + 2);

  MixedState h{};
  h.max_iter = max_iter;
  h.norm_b = op->norm_b;
  h.tol_norm_b = mp.tol * op->norm_b;
  h.delta = mp.reliable_delta > 0.0 ? mp.reliable_delta : 1e-4;
  h.pad = 1;  // "x0 is zero" flag, cleared by k_is_zero
  // the state goes up and comes back through pinned memory (a pageable copy
  // can wait for the stream)
  f.h_state.alloc(1);
  *f.h_state.p = h;
  DS_CUDA(cudaMemcpyAsync(f.state.p, f.h_state.p, sizeof(h), cudaMemcpyHostToDevice, st));
  MixedState* S = f.state.p;
  int* xzero = &S->pad;

  cudaEvent_t ev0, ev1;
  DS_CUDA(cudaEventCreate(&ev0));
  DS_CUDA(cudaEventCreate(&ev1));
  DS_CUDA(cudaEventRecord(ev0, st));

  const int g = vgrid(np);
  // With the structured inner operator (skewers on one z grid) the whole
  // solve runs in record order: the structured kernels and the cluster
  // preconditioner then read and write whole skewers' runs of the vectors
  // instead of scattered sorted positions.  X, B, PD and POS are the
  // solution, right-hand side, Jacobi diagonal and record -> index map of the
  // order in use; x is converted in at the start and out at the end.
  const bool use_sg = op->sgrid && (op->inner_variant == INNER_AUTO ||
                                    op->inner_variant == INNER_STRUCTURED);
  if (!use_sg) ensure_f32_pairs(op);
  SkewerVecs sv{};
  double* X = op->x.p;
  const double* B = op->b.p;
  const float* PD = f.pdiag.p;
  const int* POS = op->inv.p;
  if (use_sg) {
    ensure_skewer_inner(op, mp.inner_cutoff > 0.0 ? mp.inner_cutoff
                                                  : DS_DEFAULT_STRUCTURED_INNER_CUTOFF);
    sv = skewer_vecs_rec(op, f.pdiag.p);
    X = op->sgrid->rx.p;
    B = sv.b;
    PD = op->sgrid->rpd.p;
    POS = nullptr;
    skewer_x_to_rec(op, op->x.p, X, st);
    // q is written on the records' indices only: its padding is cleared here
    DS_CUDA(cudaMemsetAsync(f.q.p, 0, np * sizeof(float), st));
  } else if (op->sgrid) {
    sv = skewer_vecs_sorted(op);
  }
  // r64 = b - A x0: nothing when x0 == 0 (then r64 = b); else first with the
  // FP32 operator, then FP64-accurate only when that one is near tol.
  // the structured FP64 residual writes the records' indices only: the
  // padding of r64 is cleared here, before anything writes r64
  if (op->sgrid) DS_CUDA(cudaMemsetAsync(op->r.p, 0, np * sizeof(double), st));
  k_is_zero<<<g, VB, 0, st>>>(np, X, xzero);
  DS_CHECK_LAUNCH();
  k_x_to_f32<<<g, VB, 0, st>>>(np, xzero, X, f.p.p);
  DS_CHECK_LAUNCH();
  if (use_sg) {
    skewer_product_f32(op, sv, f.p.p, f.q.p, nullptr, nullptr, nullptr, nullptr, xzero, st);
  } else {
    F32Args a0 = op_f32_args(op, f.p.p, f.q.p);
    a0.skip_flag = xzero;
    launch_pair_f32(f.formula, EPI_PRODUCT, a0, st);
  }
  k_r32_init<<<g, VB, 0, st>>>(np, S, xzero, B, f.q.p, op->r.p, op->partial.p);
  DS_CHECK_LAUNCH();
  // the structured residual takes only v, out and the skip flag: no pair list
  auto residual_args = [&](const double* v, double* out) {
    if (!op->sgrid) return op_pair_args(op, v, out);
    PairArgs pa{};
    pa.v = v;
    pa.out = out;
    return pa;
  };
  PairArgs resid = residual_args(X, op->r.p);
  resid.skip_flag = &S->init_skip;
  auto outer_residual = [&](const PairArgs& pa) {
    if (op->sgrid)
      skewer_apply_f64(op, sv, true, pa.v, pa.out, pa.skip_flag, st);
    else if (f.use_ff)
      launch_pair_ff_resid(op->kc, pa, f.ffd.view, st);
    else
      launch_pair_f64(op->kc, EPI_RESIDUAL, pa, st);
  };
  outer_residual(resid);
  const SkewerPC* pc = op->pc.get();
  PcArgs pa0{};
  if (pc) {
    pa0.n_slots = pc->n_sk * pc->n_per;
    pa0.band = pc->band;
    pa0.st = S;
    pa0.x_zero = xzero;
    pa0.crec = pc->crec.p;
    pa0.inv = POS;
    pa0.L = pc->L.p;
    pa0.x = X;
    pa0.z = f.z.p;
    pa0.p = f.p.p;
    pa0.hist = f.hist.p;
    pa0.htrue = f.htrue.p;
  }
  // partial2 holds the p.q partials of K1 (one per row tile) and, in the
  // preconditioned form, the (r.z, |r|^2) partials per skewer after them.
  double* pc_part = op->partial2.p + op->pix.n_tiles;
  // the band preconditioner updates r out of place: iteration it reads
  // rbuf[(it - 1) & 1] and writes rbuf[it & 1] (the start writes rbuf[0])
  float* rbuf[2] = {f.r.p, nullptr};
  if (pc) {
    f.r2.alloc(np);
    rbuf[1] = f.r2.p;
    // padding stays 0 in every FP32 vector
    for (float* v : {f.z.p, f.r.p, f.r2.p, f.p.p})
      DS_CUDA(cudaMemsetAsync(v, 0, np * sizeof(float), st));
    PcArgs a = pa0;
    a.rout = rbuf[0];
    a.b = B;
    a.r64 = op->r.p;
    a.part = pc_part;
    pc_iter<2>(a, st);
  } else {
    k_mx_init<<<g, VB, 0, st>>>(np, S, xzero, B, op->r.p, f.r.p, f.z.p, f.p.p, PD,
                                op->partial.p, f.hist.p, f.htrue.p);
    DS_CHECK_LAUNCH();
  }

  F32Args prod = op_f32_args(op, f.p.p, f.q.p);
  prod.dotv = f.p.p;
  prod.dot_partial = op->partial2.p;
  prod.counter = &S->counter[0];
  prod.num = &S->rz;
  prod.alpha_out = &S->alpha;
  prod.den_out = &S->pq;
  prod.skip_flag = &S->done;
  PairArgs upd = residual_args(X, op->r.p);
  upd.skip_flag = &S->skip_update;
  if (!f.tc_err.p) {
    f.tc_err.alloc(1);
    DS_CUDA(cudaMemsetAsync(f.tc_err.p, 0, sizeof(int), st));
  }
  prod.err = f.tc_err.p;
  if (op->inner_variant == INNER_TENSOR && f.formula == F32_EXPANDED && !f.tc_cols.p)
    f.tc_cols.alloc((size_t)np * 16);
  prod.tc_cols = f.tc_cols.p;
  // The CUDA-core kernel is the default: on GB300 it measures 0.22 ms per
  // product on the 262,144-pixel workload against 0.36 ms for the tensor-core
  // kernel (whose consumers wait on TMEM-load and MMA latency with only two
  // T / S buffers in the 512 TMEM columns).
  const bool use_tc =
      op->inner_variant == INNER_TENSOR && pair_tc_usable(f.formula, EPI_PRODUCT, prod);

  // One iteration: K1 (q = A32 p, p.q, alpha), K2 (x, r updates, z = M^-1 r,
  // r.z, update test), K5 (FP64-accurate residual when an update is due),
  // K6 (the update), K7 (p = z + beta p).  Every kernel returns at once once
  // the solve is done, so iterations launched past the end change nothing.
  auto iteration = [&](int it) {
    if (use_sg)
      // K7 of the previous iteration (p = z + beta p) is done by K1 here
      skewer_product_f32(op, sv, f.p.p, prod.out, prod.counter, prod.num, prod.alpha_out,
                         prod.den_out, prod.skip_flag, st, &S->beta, f.z.p);  // K1
    else if (use_tc)
      launch_pair_tc(prod, st);                                               // K1
    else
      launch_pair_f32(f.formula, EPI_PRODUCT, prod, st);
    if (pc) {
      PcArgs a = pa0;                                                         // K2
      a.rin = rbuf[(it - 1) & 1];
      a.rout = rbuf[it & 1];
      a.q = f.q.p;
      a.part = pc_part;
      pc_iter<0>(a, st);
    } else {
      k_mx_update<<<g, VB, 0, st>>>(np, S, X, f.r.p, f.z.p, f.p.p, f.q.p, PD, op->partial.p,
                                    f.hist.p);                               // K2
      DS_CHECK_LAUNCH();
    }
    outer_residual(upd);                                                      // K5
    if (pc) {
      PcArgs a = pa0;                                                         // K6
      a.rout = rbuf[it & 1];
      a.r64 = op->r.p;
      a.part = pc_part;
      pc_iter<1>(a, st);
    } else {
      k_mx_replace<<<g, VB, 0, st>>>(np, S, op->r.p, f.r.p, f.z.p, PD, op->partial.p, f.hist.p,
                                     f.htrue.p);                             // K6
      DS_CHECK_LAUNCH();
    }
    if (!use_sg) {
      k_mx_dir<<<g, VB, 0, st>>>(np, S, f.z.p, f.p.p);                      // K7
      DS_CHECK_LAUNCH();
    }
  };

  // The host reads the done flag every CHECK iterations, two reads behind,
  // so the stream never drains.  Without profiling (and with the CUDA-core or
  // structured inner product) the CHECK iterations are one CUDA graph,
  // captured once per solve and replayed: 1 launch instead of ~7 CHECK.
  constexpr int CHECK = 8;
  constexpr int NSLOT = 64;
  cudaEvent_t evs[NSLOT] = {};
  cudaGraphExec_t gexec = nullptr;
  long long per_graph = 0;
  // With the structured inner operator and a band preconditioner the whole
  // loop can be one cooperative launch (persist.cu); profiling keeps the
  // per-kernel form, whose kernels it times one by one.
  bool persisted = false;
  if (use_sg && pc && op->iter_form == DS_ITER_AUTO && !op->ctx->prof.enabled && max_iter > 0)
    persisted = run_mixed_persistent(op, f, pc, sv, X, rbuf[0], max_iter, st);
  if (!persisted)  // the host polls the done flag (the persistent launch needs no events)
    for (auto& e : evs) DS_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  if (!persisted && !op->ctx->prof.enabled && !use_tc && max_iter > 0) {
    const long long l0 = launch_counter();
    cudaGraph_t graph = nullptr;
    DS_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    try {
      for (int k = 1; k <= CHECK; ++k) iteration(k);  // CHECK is even: parities repeat
    } catch (...) {
      cudaStreamEndCapture(st, &graph);
      if (graph) cudaGraphDestroy(graph);
      throw;
    }
    DS_CUDA(cudaStreamEndCapture(st, &graph));
    const cudaError_t inst = cudaGraphInstantiate(&gexec, graph, 0);
    cudaGraphDestroy(graph);
    DS_CUDA(inst);
    per_graph = launch_counter() - l0;
  }
  int issued = 0, waited = 0, replays = 0;
  for (int it = 1; !persisted && it <= max_iter; it += gexec ? CHECK : 1) {
    if (gexec) {
      DS_CUDA(cudaGraphLaunch(gexec, st));
      ++replays;
    } else {
      iteration(it);
    }
    if (gexec || it % CHECK == 0) {
      const int slot = issued % NSLOT;
      DS_CUDA(cudaMemcpyAsync(&op->h_flag.p[slot], &S->done, sizeof(int),
                              cudaMemcpyDeviceToHost, st));
      DS_CUDA(cudaEventRecord(evs[slot], st));
      ++issued;
      if (issued - waited > 2) {
        const int ws = waited % NSLOT;
        DS_CUDA(cudaEventSynchronize(evs[ws]));
        ++waited;
        if (op->h_flag.p[ws]) break;
      }
    }
  }
  if (gexec) {
    // the capture counted one graph's launches; each further replay launches them again
    launch_counter() += (long long)std::max(replays - 1, 0) * per_graph;
    cudaGraphExecDestroy(gexec);
  }
  if (use_sg) skewer_x_to_sorted(op, X, op->x.p, st);
  DS_CUDA(cudaEventRecord(ev1, st));
  DS_CUDA(cudaMemcpyAsync(f.h_state.p, S, sizeof(h), cudaMemcpyDeviceToHost, st));
  DS_CUDA(cudaStreamSynchronize(st));
  h = *f.h_state.p;
  float ms = 0.f;
  DS_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
  for (auto& e : evs)
    if (e) cudaEventDestroy(e);
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);

  if (persisted) {
    const int code = persistent_error(op, st);
    if (code)
      throw Error{DS_ERR_TIMEOUT, "persistent mixed solve: a grid barrier wait timed out "
                                  "(phase " + std::to_string(code) + ")"};
  }
  if (use_tc) {
    int code = 0;
    DS_CUDA(cudaMemcpyAsync(&code, f.tc_err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    DS_CUDA(cudaStreamSynchronize(st));
    if (code) {
      DS_CUDA(cudaMemsetAsync(f.tc_err.p, 0, sizeof(int), st));
      throw Error{DS_ERR_CUDA, "tensor-core inner matvec: an mbarrier wait timed out (code " +
                                   std::to_string(code) + ")"};
    }
  }
  const int n_hist = h.iter + 1;
  if (hist_out)
    DS_CUDA(cudaMemcpyAsync(hist_out, f.hist.p, n_hist * sizeof(double), cudaMemcpyDeviceToHost, st));
  DS_CUDA(cudaStreamSynchronize(st));
  res.norm_b = op->norm_b;
  res.final_norm = h.rtrue;
  res.seconds = ms * 1e-3;
  res.n_outer = h.n_updates;
  res.n_inner = h.iter;
  res.num_iters = h.iter;
  res.success = h.converged;
  if (mp.verbose) {
    std::vector<double> ht(h.n_updates + 1);
    DS_CUDA(cudaMemcpyAsync(ht.data(), f.htrue.p, ht.size() * sizeof(double),
                       cudaMemcpyDeviceToHost, st));
    DS_CUDA(cudaStreamSynchronize(st));
    printf("[PCG mixed] %d FP32 iterations, %d FP64 residual updates, |r| %e (tol |b| %e)\n",
           h.iter, h.n_updates, h.rtrue, h.tol_norm_b);
    for (size_t k = 0; k < ht.size(); ++k) printf("    update %zu: |r| = %e\n", k, ht[k]);
  }
}

void ensure_map_f32(ds_map* map, ds_operator* op, double cut) {
  ensure_map_points(map);
  if (map->f32 && map->f32->op_serial == op->serial && map->f32->cut == cut) return;
  cudaStream_t st = map->ctx->stream;
  std::unique_ptr<MapF32, MapF32Deleter> f(new MapF32());
  f->op_serial = op->serial;
  f->cut = cut;
  double sp, sq;
  exact_scales(op->kc, sp, sq);
  build_f32_points(f->pts, map->pts, sp, sp, sq, st);
  KernelConsts kc = op->kc;
  kc.cull_arg = cut * (1.0 + 1e-9);
  build_pair_list(f->pairs, map->pts, op->pix, kc, st);
  build_slice_items(f->pairs, st);
  f->rowf.alloc(map->pts.n_pad);
  k_fill_f32<<<vgrid(map->pts.n_pad), VB, 0, st>>>(map->pts.n_pad, (float)op->kc.var_s,
                                                   f->rowf.p);
  DS_CHECK_LAUNCH();
  f->xs.alloc(op->pix.n_pad);
  DS_CUDA(cudaStreamSynchronize(st));
  map->f32 = std::move(f);
}

// m = S_mp x with FP32 kernel evaluation and FP64 accumulation across tiles.
void map_product_f32_dev(ds_map* map, ds_operator* op, const double* x_dev, double* m_dev,
                         double cut) {
  require(op->kc.eval == DS_EVAL_EXACT, "the FP32 map product evaluates the exact kernel");
  // a column-grid map against a skewer grid: the structured FP64 product
  if (skewer_map_product(map, op, x_dev, m_dev, cut)) return;
  ensure_op_f32(op, op->f32 ? op->f32->inner_cut : DS_DEFAULT_INNER_CUTOFF);
  ensure_map_f32(map, op, cut);
  cudaStream_t st = map->ctx->stream;
  MapF32& f = *map->f32;
  op->tmp.alloc(op->pix.n_pad);
  gather_sorted(op->pix, x_dev, op->tmp.p, st);
  k_d2f<<<vgrid(op->pix.n_pad), VB, 0, st>>>(op->pix.n_pad, op->tmp.p, f.xs.p);
  DS_CHECK_LAUNCH();
  F32Args a{};
  a.rxi = f.pts.xi.p;
  a.rorig = f.pts.orig.p;
  a.cxi = op->f32->pts.xi.p;
  a.corig = op->f32->pts.orig.p;
  a.row_ptr = f.pairs.row_ptr.p;
  a.cols = f.pairs.cols.p;
  a.mask = f.pairs.mask.p;
  a.item_ptr = f.pairs.item_ptr.p;
  a.items = f.pairs.items.p;
  a.row_order = f.pairs.row_order.p;
  a.n_row_tiles = map->pts.n_tiles;
  a.v = f.xs.p;
  a.rowf = f.rowf.p;
  a.row_perm = map->pts.perm.p;
  a.out64 = m_dev;
  a.n_tile_pairs = f.pairs.n_pairs;
  a.prof = &map->ctx->prof;
  launch_pair_f32(F32_DIRECT, EPI_MAP, a, st);
}

}  // namespace ds
