// Float-float ("double-single") arithmetic for an FP64-accurate evaluation of
// the exact kernel on the FP32 pipe.  GB300 issues FP64 at 2 operations per
// clock per SM against 128 FP32 lanes, so the FP64-accurate outer residual
// of the mixed-precision solver evaluates
//     S_ij / var_s = exp(-(dX^2 + dY^2 + dZ^2))
// (coordinates scaled by sqrt(c_perp), sqrt(c_para)) with unevaluated float
// pairs (hi + lo, about 48 significant bits), following the published
// error-free transformations (Knuth's two-sum, Dekker's fast two-sum, the
// FMA-based exact product).  Every operation below rounds exactly as written:
// the __f*_rn intrinsics keep the compiler from contracting or reassociating
// them.
#pragma once

#include <cuda_runtime.h>

namespace ds {

struct ff {
  float h, l;
};

// s + e = a + b exactly (Knuth).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// s + e = a + b exactly when |a| >= |b| (Dekker).
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

// a - b for float pairs, renormalised.
__device__ __forceinline__ ff ff_sub(ff a, ff b) {
  float s, e;
  two_sum(a.h, -b.h, s, e);
  e = __fadd_rn(e, __fsub_rn(a.l, b.l));
  ff r;
  fast_two_sum(s, e, r.h, r.l);
  return r;
}

// a^2 (not renormalised; the lo part drops a.l^2).
__device__ __forceinline__ ff ff_sqr(ff a) {
  ff r;
  r.h = __fmul_rn(a.h, a.h);
  r.l = __fmaf_rn(a.h, a.h, -r.h);
  r.l = __fmaf_rn(__fadd_rn(a.h, a.h), a.l, r.l);
  return r;
}

// a + b for float pairs, renormalised.
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  e = __fadd_rn(e, __fadd_rn(a.l, b.l));
  ff r;
  fast_two_sum(s, e, r.h, r.l);
  return r;
}

// |dX|^2 for the three scaled coordinate differences Y - X.
__device__ __forceinline__ ff ff_dist2(ff yx, ff yy, ff yz, ff xx, ff xy, ff xz) {
  const ff dx = ff_sub(yx, xx), dy = ff_sub(yy, xy), dz = ff_sub(yz, xz);
  return ff_add(ff_add(ff_sqr(dx), ff_sqr(dy)), ff_sqr(dz));
}

// exp(-a) for 0 <= a < 60 as a float pair (relative error about 1e-14),
// written from the mathematics:
//   k = round(32 a / ln 2),  r = a - k ln2/32 (|r| <= ln2/64; ln2/32 split
//   into a 12-bit head, so that k * head is exact for k < 4096, and two
//   tails), exp(-a) = 2^-(k >> 5) * 2^-((k & 31) / 32) * exp(-r);
// exp(-r) = 1 - r + r^2/2 + T with the r^2/2 term and the leading terms in
// float pairs and T = -r^3/6 + ... + r^6/720 in FP32 (|T| < 2.2e-7, so its
// FP32 rounding stays below 2e-14); 2^-(j/32) from a 32-entry table of float
// pairs ``tab_h``, ``tab_l``; the power of two applied exactly.
__device__ __forceinline__ ff ff_exp_neg(ff a, const float* tab_h, const float* tab_l) {
  const float M = 12582912.f;  // 1.5 * 2^23: rounds to an integer in the low bits
  const float K32_LN2 = 46.16624069213867f;
  const float C_HI = 0.02165985107421875f;     // ln2/32, 12 significant bits
  const float C_MID = 9.983182280848268e-07f;
  const float C_LO = 5.145536774442405e-14f;
  const float t = __fmaf_rn(a.h, K32_LN2, M);
  const int k = __float_as_int(t) - __float_as_int(M);
  const float kf = __fsub_rn(t, M);
  // r = a - k C, as a float pair
  const float r1 = __fmaf_rn(-kf, C_HI, a.h);  // exact (Sterbenz)
  const float pm = __fmul_rn(kf, C_MID);
  const float pm_e = __fmaf_rn(kf, C_MID, -pm);
  float rh, re;
  two_sum(r1, -pm, rh, re);
  re = __fadd_rn(re, __fsub_rn(a.l, __fmaf_rn(kf, C_LO, pm_e)));
  float sh, sl;  // s = -r
  fast_two_sum(rh, re, sh, sl);
  sh = -sh;
  sl = -sl;
  // exp(s) = 1 + s + s^2/2 + T
  const float s2 = __fmul_rn(sh, sh);
  const float s3 = __fmul_rn(s2, sh);
  float poly = __fmaf_rn(sh, 1.f / 720.f, 1.f / 120.f);
  poly = __fmaf_rn(sh, poly, 1.f / 24.f);
  poly = __fmaf_rn(sh, poly, 1.f / 6.f);
  const float T = __fmul_rn(s3, poly);
  const float qh = __fmul_rn(0.5f, s2);
  const float ql = __fmul_rn(0.5f, __fmaf_rn(__fadd_rn(sh, sh), sl, __fmaf_rn(sh, sh, -s2)));
  float h1, e1, h2, e2;
  fast_two_sum(1.f, sh, h1, e1);
  fast_two_sum(h1, qh, h2, e2);
  const float lo = __fadd_rn(__fadd_rn(__fadd_rn(e1, e2), __fadd_rn(sl, ql)), T);
  float eh, el;
  fast_two_sum(h2, lo, eh, el);
  // times 2^-(j/32)
  const int j = k & 31;
  const float th = tab_h[j], tl = tab_l[j];
  const float ph = __fmul_rn(eh, th);
  float pl = __fmaf_rn(eh, th, -ph);
  pl = __fmaf_rn(eh, tl, pl);
  pl = __fmaf_rn(el, th, pl);
  // times 2^-(k >> 5), exact (no underflow for a < 60)
  const float sc = __int_as_float((127 - (k >> 5)) << 23);
  ff r;
  r.h = __fmul_rn(ph, sc);
  r.l = __fmul_rn(pl, sc);
  return r;
}

// (ah, al) += s * u for float pairs: the product's rounding error from an
// FMA, the cross terms in FP32, Knuth's two-sum for the high part.
__device__ __forceinline__ void ff_mac(float& ah, float& al, ff s, ff u) {
  const float p = __fmul_rn(s.h, u.h);
  float e = __fmaf_rn(s.h, u.h, -p);
  e = __fmaf_rn(s.h, u.l, e);
  e = __fmaf_rn(s.l, u.h, e);
  float t, err;
  two_sum(ah, p, t, err);
  al = __fadd_rn(al, __fadd_rn(err, e));
  ah = t;
}

// x (FP64) as a float pair.
__device__ __forceinline__ ff ff_from_double(double x) {
  ff r;
  r.h = __double2float_rn(x);
  r.l = __double2float_rn(x - (double)r.h);
  return r;
}

}  // namespace ds
