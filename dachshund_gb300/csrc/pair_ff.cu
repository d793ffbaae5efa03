// FP64-accurate residual r = b - A x of the exact-kernel operator on the FP32
// pipe (float-float arithmetic, ds_ff.cuh): the outer residual of the
// mixed-precision solver (the reliable updates and its stopping test).
// Same tiling as the FP64 pair kernel (k_pair_f64): one CTA per row tile, one
// row per thread, warp-private staging of the column sub-tiles the warp's
// rows interact with.
//
// Coordinates: every pixel carries its coordinates scaled by sqrt(c_perp),
// sqrt(c_para) and taken relative to its own tile's origin, as float pairs
// (fx, fy, fz); for each tile pair a row thread forms its own scaled
// coordinates relative to the column tile's origin in FP64 once and splits
// them, so that the per-pair differences are float-pair subtractions of
// numbers of a few correlation lengths.  Per pair: about 64 FP32 operations
// for the argument, 46 for exp, 12 for the float-pair multiply-add, against
// about 20 FP64 operations (at 1/64 of the FP32 rate) in k_pair_f64.
//
// Far pairs: a term with argument >= FF_FAR (16) is at most e^-16 = 1.1e-7
// of var_s |u_j|, and FP32 evaluation gets its argument to ~2e-6 absolute
// (coordinates differenced from float pairs), i.e. the term to ~2e-6
// relative: an absolute error near 2e-13 of var_s |u_j| per term.  For each
// column the warp first forms the FP32 argument of its 32 rows; when all of
// them are >= FF_FAR the column's terms are evaluated in FP32 (one MUFU ex2,
// accumulated apart), else by the float-pair path.  Between argument 16 and
// the operator's cutoff (40 by default) lie about three quarters of the
// pairs this residual evaluates.  Measured on the 262,144-pixel system: the
// residual stays within 4e-12 relative of the FP64 residual, as with the
// threshold at 24 (where the FP32 path took half the pairs), while the
// residual takes 3.3 ms instead of 4.1.
#include <cmath>

#include "ds_device.cuh"
#include "ds_f32.h"
#include "ds_ff.cuh"

namespace ds {

namespace {

constexpr float FF_FAR = 16.f;                   // FP32 evaluation at or beyond this argument
constexpr float LOG2E_F = 1.4426950408889634f;   // log2(e)

__device__ __forceinline__ float ex2_ff(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Scaled tile-relative float-pair coordinates and the scaled tile origins.
__global__ void k_ff_points(int n_pad, const double* __restrict__ x, const double* __restrict__ y,
                            const double* __restrict__ z, const double* __restrict__ box,
                            double sp, double sq, float2* __restrict__ fx,
                            float2* __restrict__ fy, float2* __restrict__ fz,
                            double* __restrict__ orig) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_pad) return;
  const int t = i / TILE;
  const double* b = box + (size_t)t * 6;
  const double ox = 0.5 * (b[0] + b[3]) * sp, oy = 0.5 * (b[1] + b[4]) * sp;
  const double oz = 0.5 * (b[2] + b[5]) * sq;
  const ff X = ff_from_double(x[i] * sp - ox), Y = ff_from_double(y[i] * sp - oy);
  const ff Z = ff_from_double(z[i] * sq - oz);
  fx[i] = make_float2(X.h, X.l);
  fy[i] = make_float2(Y.h, Y.l);
  fz[i] = make_float2(Z.h, Z.l);
  if (i % TILE == 0) {
    orig[3 * t + 0] = ox;
    orig[3 * t + 1] = oy;
    orig[3 * t + 2] = oz;
  }
}

__global__ void __launch_bounds__(TILE) k_pair_ff_resid(KernelConsts kc, PairArgs a, FFPoints f) {
  if (a.skip_flag && *a.skip_flag) return;
  __shared__ float sw[TILE / 32][8][SUBTILE];  // xh xl yh yl zh zl uh ul
  __shared__ float tab_h[32], tab_l[32];
  const int t = a.row_order ? a.row_order[blockIdx.x] : blockIdx.x;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int i = t * TILE + tid;
  if (tid < 32) {
    const ff v = ff_from_double(exp2(-(double)tid / 32.0));
    tab_h[tid] = v.h;
    tab_l[tid] = v.l;
  }
  __syncthreads();
  const float cut = (float)kc.exact_cut;
  const double xi = a.rx[i] * f.sp, yi = a.ry[i] * f.sp, zi = a.rz[i] * f.sq;
  float ah = 0.f, al = 0.f;
  float af = 0.f;  // far terms (FP32)
  unsigned long long evaluated = 0;
  float* s = &sw[warp][0][0];
  const int p0 = a.row_ptr[t], p1 = a.row_ptr[t + 1];
  for (int p = p0; p < p1; ++p) {
    const unsigned m = (a.mask[p] >> (4 * warp)) & 0xFu;
    if (!m) continue;
    const int ct = a.cols[p];
    // this row relative to the column tile's origin
    const ff Yx = ff_from_double(xi - f.orig[3 * ct + 0]);
    const ff Yy = ff_from_double(yi - f.orig[3 * ct + 1]);
    const ff Yz = ff_from_double(zi - f.orig[3 * ct + 2]);
    for (int cs = 0; cs < TILE / SUBTILE; ++cs) {
      if (!((m >> cs) & 1u)) continue;
      const int j = ct * TILE + cs * SUBTILE + lane;
      __syncwarp();
      const float2 cx = f.fx[j], cy = f.fy[j], cz = f.fz[j];
      const ff u = ff_from_double(kc.var_s * (a.wr[j] * a.v[j]));
      s[0 * SUBTILE + lane] = cx.x;
      s[1 * SUBTILE + lane] = cx.y;
      s[2 * SUBTILE + lane] = cy.x;
      s[3 * SUBTILE + lane] = cy.y;
      s[4 * SUBTILE + lane] = cz.x;
      s[5 * SUBTILE + lane] = cz.y;
      s[6 * SUBTILE + lane] = u.h;
      s[7 * SUBTILE + lane] = u.l;
      __syncwarp();
      evaluated += SUBTILE * SUBTILE;
#pragma unroll 2
      for (int jj = 0; jj < SUBTILE; ++jj) {
        const ff X{s[0 * SUBTILE + jj], s[1 * SUBTILE + jj]};
        const ff Y{s[2 * SUBTILE + jj], s[3 * SUBTILE + jj]};
        const ff Z{s[4 * SUBTILE + jj], s[5 * SUBTILE + jj]};
        const float dx = (Yx.h - X.h) + (Yx.l - X.l);
        const float dy = (Yy.h - Y.h) + (Yy.l - Y.l);
        const float dz = (Yz.h - Z.h) + (Yz.l - Z.l);
        const float d2f = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        if (__all_sync(0xffffffffu, d2f >= FF_FAR)) {
          if (d2f < cut) af = fmaf(ex2_ff(-d2f * LOG2E_F), s[6 * SUBTILE + jj], af);
        } else {
          const ff d2 = ff_dist2(Yx, Yy, Yz, X, Y, Z);
          if (d2.h < cut) {
            const ff g = ff_exp_neg(d2, tab_h, tab_l);
            ff_mac(ah, al, g, ff{s[6 * SUBTILE + jj], s[7 * SUBTILE + jj]});
          }
        }
      }
    }
  }
  if (a.prof_pairs && lane == 0) atomicAdd(a.prof_pairs, evaluated);
  const double acc = ((double)ah + (double)al) + (double)af;
  a.out[i] = a.b[i] - (a.wl[i] * acc + a.e[i] * a.v[i]);
}

}  // namespace

bool ff_usable(const KernelConsts& kc) {
  // exp(-a) of ff_exp_neg stays a normal float pair for a < 60
  return kc.eval == DS_EVAL_EXACT && kc.exact_cut <= 60.0;
}

void build_ff_points(FFData& f, const PointSet& ps, const KernelConsts& kc, cudaStream_t st) {
  const double sp = std::sqrt(kc.c_perp), sq = std::sqrt(kc.c_para);
  f.fx.alloc(ps.n_pad);
  f.fy.alloc(ps.n_pad);
  f.fz.alloc(ps.n_pad);
  f.orig.alloc((size_t)3 * ps.n_tiles);
  k_ff_points<<<(ps.n_pad + 255) / 256, 256, 0, st>>>(ps.n_pad, ps.x.p, ps.y.p, ps.z.p, ps.box.p,
                                                      sp, sq, f.fx.p, f.fy.p, f.fz.p, f.orig.p);
  DS_CHECK_LAUNCH();
  f.view.fx = f.fx.p;
  f.view.fy = f.fy.p;
  f.view.fz = f.fz.p;
  f.view.orig = f.orig.p;
  f.view.sp = sp;
  f.view.sq = sq;
}

// r = b - A v (FP64-accurate, float-float evaluation); profiled as an FP64
// kernel (kind 0).
void launch_pair_ff_resid(const KernelConsts& kc, const PairArgs& a0, const FFPoints& f,
                          cudaStream_t st) {
  if (a0.n_row_tiles <= 0) return;
  PairArgs a = a0;
  cudaEvent_t ev = nullptr;
  if (a.prof && a.prof->enabled) {
    a.prof_pairs = a.prof->d_pairs;
    a.prof->begin(st, &ev);
  } else {
    a.prof_pairs = nullptr;
  }
  k_pair_ff_resid<<<a.n_row_tiles, TILE, 0, st>>>(kc, a, f);
  DS_CHECK_LAUNCH();
  if (ev) a.prof->end(st, ev, 0);
}

}  // namespace ds
