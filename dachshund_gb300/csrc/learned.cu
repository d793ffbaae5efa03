// Learned warm start and per-skewer preconditioner (no reference
// counterpart): a small message-passing network over the pixels of a
// skewer-structured pixel set (n_sk skewers of n_per pixels sharing one
// z grid, records skewer-contiguous) predicts, for the W-form system
// (I + w S w) y = w d,
//   * a warm start y0 for the solve, and
//   * per skewer a lower-triangular band factor L (bandwidth B, positive
//     diagonal), the preconditioner M^-1 = L L^T of that skewer's block.
// Forward, backward and optimiser are the kernels below (CUDA cores, FP32
// arithmetic on BF16 weights); the tensor cores are left to the batched
// S-tile x RHS matvec.
//
// Network (hidden width H, F_IN = 11 inputs per pixel):
//   inputs   z position along the skewer, log noise, the whitened datum w d,
//            and g_n = exp(-dperp_n^2 / (2 l_perp^2)) to the 8 nearest
//            neighbour skewers;
//   embed    h0 = relu(X W_in + b_in);
//   layers   h_l = h_{l-1} + relu([h | A_z h | A_n h] W_l + b_l), l = 1..4,
//            A_z h_i = h_{i-1} + h_{i+1} along the skewer, A_n h_i =
//            sum_n g_n h_{(neighbour n, same z index)};
//   head     Y = h_4 W_o + b_o (2 + B outputs per pixel):
//            y0 = XS Y_0,
//            L_ii = exp(SD tanh(Y_1)) / sqrt(1 + w_i^2 var_s)  (the Jacobi
//            factor times a learned factor in [e^-SD, e^SD]: the network
//            starts from Jacobi-PCG and cannot collapse L to 0, where the
//            quartic loss below is stationary),
//            L_{i,i-1} = a1 L_ii, L_{i,i-2} = a2 L_ii (band B = 2, inside the
//            skewer) with a2 = AC tanh(Y_3), a1 = AC (1 + a2) tanh(Y_2): each
//            row's polynomial 1 + a1 z + a2 z^2 lies inside the stability
//            triangle (|a2| < 1, |a1| < 1 + a2), so that L^-1 does not grow
//            along a 256-pixel skewer (free band coefficients can make
//            L L^T numerically singular).
// Losses (trained on solutions of the plain solver):
//   warm start     sum (y0 - y*)^2 / sum y*^2;
//   preconditioner per skewer, with probe vectors v:
//                  sum |L L^T A_bb v - v|^2 / n, A_bb the skewer's own block
//                  of I + w S w (its pixels only).
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "ds_f32.h"
#include "ds_learned.h"
#include "ds_ops.h"

namespace ds {
namespace {

constexpr int NB_K = 8;   // neighbour skewers
constexpr float XS = 0.3f, SD = 1.0f, AC = 0.9f;
constexpr float LOGN0 = -2.1f, LOGNS = 0.6f;  // log-noise normalisation

inline unsigned grid1(size_t n, int nt = 256) { return (unsigned)((n + nt - 1) / nt); }


// ---- geometry and inputs --------------------------------------------------------

// (x, y) of every skewer (its first record) in one compact array.
__global__ void k_skewer_xy(int n_sk, int n_per, const double* __restrict__ rec,
                            double2* __restrict__ xy) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n_sk) xy[s] = make_double2(rec[(size_t)s * n_per * 5], rec[(size_t)s * n_per * 5 + 1]);
}

// The 8 nearest skewers of every skewer (brute force over the skewer (x, y)),
// with weights g = exp(-d^2 / (2 l_perp^2)); nearer first, ties by index, the
// missing ones (fewer than 9 skewers) pointing at the skewer itself with
// g = 0.  One warp per skewer: lane l keeps the 8 nearest of skewers
// l, l + 32, ... in order, then 8 rounds of a warp minimum over the lanes'
// heads merge them.
__global__ void k_knn(int n_sk, const double2* __restrict__ xy, double inv2l2,
                      int* __restrict__ nbr, float* __restrict__ g) {
  const int s = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (s >= n_sk) return;  // warp-uniform
  const double2 ps = xy[s];
  double bd[NB_K];
  int bi[NB_K];
#pragma unroll
  for (int k = 0; k < NB_K; ++k) {
    bd[k] = 1e300;
    bi[k] = s;
  }
  for (int o = lane; o < n_sk; o += 32) {
    if (o == s) continue;
    const double2 q = xy[o];
    const double dx = q.x - ps.x, dy = q.y - ps.y;
    const double d2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
    if (d2 >= bd[NB_K - 1]) continue;  // o only grows: an equal d2 stays behind
    // insertion after every entry <= d2 (static indices only)
    bool placed = false;
#pragma unroll
    for (int k = NB_K - 1; k > 0; --k) {
      if (!placed) {
        if (bd[k - 1] > d2) {
          bd[k] = bd[k - 1];
          bi[k] = bi[k - 1];
        } else {
          bd[k] = d2;
          bi[k] = o;
          placed = true;
        }
      }
    }
    if (!placed) {
      bd[0] = d2;
      bi[0] = o;
    }
  }
  constexpr unsigned full = 0xffffffffu;
  double od[NB_K];
  int oi[NB_K];
#pragma unroll
  for (int r = 0; r < NB_K; ++r) {
    double d = bd[0];
    int idx = bi[0], who = lane;
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) {
      const double d2 = __shfl_xor_sync(full, d, m);
      const int i2 = __shfl_xor_sync(full, idx, m), w2 = __shfl_xor_sync(full, who, m);
      if (d2 < d || (d2 == d && (i2 < idx || (i2 == idx && w2 < who)))) {
        d = d2;
        idx = i2;
        who = w2;
      }
    }
    od[r] = d;
    oi[r] = idx;
    if (lane == who) {  // pop the head
#pragma unroll
      for (int k = 0; k < NB_K - 1; ++k) {
        bd[k] = bd[k + 1];
        bi[k] = bi[k + 1];
      }
      bd[NB_K - 1] = 1e300;
      bi[NB_K - 1] = s;
    }
  }
  if (lane < NB_K) {
    double d = od[0];
    int idx = oi[0];
#pragma unroll
    for (int r = 1; r < NB_K; ++r)
      if (lane == r) {
        d = od[r];
        idx = oi[r];
      }
    nbr[s * NB_K + lane] = idx;
    g[s * NB_K + lane] = idx == s ? 0.f : (float)exp(-d * inv2l2);
  }
}

// Input features of every pixel (caller order: i = s n_per + k).
__global__ void k_features(int n, int n_per, const double* __restrict__ rec,
                           const float* __restrict__ g, float* __restrict__ X) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int s = i / n_per, k = i % n_per;
  const double w = rec[(size_t)i * 5 + 3], wd = rec[(size_t)i * 5 + 4];
  float* x = X + (size_t)i * F_IN;
  x[0] = n_per > 1 ? 2.f * k / (n_per - 1) - 1.f : 0.f;
  x[1] = ((float)(-log(w)) - LOGN0) / LOGNS;  // log n
  x[2] = 0.5f * (float)wd;
  for (int m = 0; m < NB_K; ++m) x[3 + m] = g[s * NB_K + m];
}

// ---- dense layers -------------------------------------------------------------------

// C[M x N] = A[M x K] B + bias, A FP32 row-major (lda), B BF16: row-major
// K x N (ldb) or, with TB, stored N x K (B(k, n) = Bm[n ldb + k]).  Epilogue
// (EPI): 0 plain store; 1 Z = C stored, out = relu(Z); 2 Z stored,
// out = res + relu(Z).  64 x 64 tiles, K steps of 16, 256 threads with 4 x 4
// outputs each.
template <bool TB, int EPI>
__global__ void __launch_bounds__(256) k_gemm(int M, int N, int K, const float* __restrict__ A,
                                              int lda, const __nv_bfloat16* __restrict__ Bm,
                                              int ldb, const float* __restrict__ bias,
                                              float* __restrict__ Z, float* __restrict__ out,
                                              const float* __restrict__ res, int ldc) {
  __shared__ float As[16][64 + 1];
  __shared__ float Bs[16][64];
  const int tid = threadIdx.x;
  const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  const int tr = tid / 16, tc = tid % 16;  // 4 rows x 4 cols each
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += 16) {
    for (int q = tid; q < 64 * 16; q += 256) {
      const int r = q / 16, kk = q % 16;
      const int m = m0 + r, k = k0 + kk;
      As[kk][r] = (m < M && k < K) ? A[(size_t)m * lda + k] : 0.f;
    }
    for (int q = tid; q < 16 * 64; q += 256) {
      const int kk = q / 64, c = q % 64;
      const int k = k0 + kk, n = n0 + c;
      float v = 0.f;
      if (k < K && n < N)
        v = __bfloat162float(TB ? Bm[(size_t)n * ldb + k] : Bm[(size_t)k * ldb + n]);
      Bs[kk][c] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        a[u] = As[kk][tr * 4 + u];
        b[u] = Bs[kk][tc * 4 + u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(a[u], b[v], acc[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int m = m0 + tr * 4 + u;
    if (m >= M) continue;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int n = n0 + tc * 4 + v;
      if (n >= N) continue;
      const float c = acc[u][v] + (bias ? bias[n] : 0.f);
      const size_t o = (size_t)m * ldc + n;
      if (EPI == 0) {
        out[o] = c;
      } else {
        Z[o] = c;
        const float r = fmaxf(c, 0.f);
        out[o] = EPI == 2 ? res[o] + r : r;
      }
    }
  }
}

// Partial products for C[K x N] = A^T D over a chunk of rows: A [M x K],
// D [M x N] FP32 row-major; each CTA (ky, nx, chunk) writes its 64 x 64 block
// of the chunk's contribution; k_reduce_chunks sums the chunks (fixed order).
constexpr int ATB_CHUNK = 2048;
__global__ void __launch_bounds__(256) k_gemm_atb(int M, int K, int N, const float* __restrict__ A,
                                                  int lda, const float* __restrict__ D, int ldd,
                                                  float* __restrict__ part) {
  __shared__ float As[16][64 + 1];
  __shared__ float Ds[16][64];
  const int tid = threadIdx.x;
  const int k0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  const int mc = blockIdx.z * ATB_CHUNK;
  const int m_end = min(M, mc + ATB_CHUNK);
  const int tr = tid / 16, tc = tid % 16;
  float acc[4][4] = {};
  for (int mm = mc; mm < m_end; mm += 16) {
    for (int q = tid; q < 16 * 64; q += 256) {
      const int r = q / 64, c = q % 64;
      const int m = mm + r;
      As[r][c] = (m < m_end && k0 + c < K) ? A[(size_t)m * lda + k0 + c] : 0.f;
      Ds[r][c] = (m < m_end && n0 + c < N) ? D[(size_t)m * ldd + n0 + c] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      float a[4], d[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        a[u] = As[r][tr * 4 + u];
        d[u] = Ds[r][tc * 4 + u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(a[u], d[v], acc[u][v]);
    }
    __syncthreads();
  }
  float* P = part + (size_t)blockIdx.z * K * N;
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int k = k0 + tr * 4 + u;
    if (k >= K) continue;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int n = n0 + tc * 4 + v;
      if (n < N) P[(size_t)k * N + n] = acc[u][v];
    }
  }
}

__global__ void k_reduce_chunks(int n_chunks, size_t len, const float* __restrict__ part,
                                float* __restrict__ out) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= len) return;
  float s = 0.f;
  for (int c = 0; c < n_chunks; ++c) s += part[(size_t)c * len + i];
  out[i] = s;
}

// Column sums of D [M x N] (bias gradients), in chunks then a fixed-order sum.
__global__ void k_colsum_part(int M, int N, const float* __restrict__ D,
                              float* __restrict__ part) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const int mc = blockIdx.y * ATB_CHUNK, me = min(M, mc + ATB_CHUNK);
  float s = 0.f;
  for (int m = mc; m < me; ++m) s += D[(size_t)m * N + n];
  part[(size_t)blockIdx.y * N + n] = s;
}

// ---- message passing ---------------------------------------------------------------

// cat_i = [h_i | h_{i-1} + h_{i+1} | sum_n g_n h_{nb_n, k}], four channels
// per thread (H % 4 == 0; 128-bit loads and stores).
__global__ void k_agg_fwd(int n, int n_per, int H, const float* __restrict__ h,
                          const int* __restrict__ nbr, const float* __restrict__ g,
                          float* __restrict__ cat) {
  const int H4 = H >> 2;
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (size_t)n * H4) return;
  const int i = (int)(q / H4), c4 = (int)(q % H4);
  const int s = i / n_per, k = i % n_per;
  const float4* h4 = reinterpret_cast<const float4*>(h);
  const float4 hi = h4[q];
  float4 az = make_float4(0.f, 0.f, 0.f, 0.f);
  if (k > 0) {
    const float4 v = h4[q - H4];
    az = make_float4(az.x + v.x, az.y + v.y, az.z + v.z, az.w + v.w);
  }
  if (k + 1 < n_per) {
    const float4 v = h4[q + H4];
    az = make_float4(az.x + v.x, az.y + v.y, az.z + v.z, az.w + v.w);
  }
  float4 an = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int m = 0; m < NB_K; ++m) {
    const float gm = g[s * NB_K + m];
    const float4 v = h4[((size_t)nbr[s * NB_K + m] * n_per + k) * H4 + c4];
    an = make_float4(fmaf(gm, v.x, an.x), fmaf(gm, v.y, an.y), fmaf(gm, v.z, an.z),
                     fmaf(gm, v.w, an.w));
  }
  float4* o = reinterpret_cast<float4*>(cat + (size_t)i * 3 * H);
  o[c4] = hi;
  o[H4 + c4] = az;
  o[2 * H4 + c4] = an;
}

// dh += adjoint of the aggregation applied to dcat (the neighbour part
// scattered with atomics: several skewers may share a neighbour).
__global__ void k_agg_bwd(int n, int n_per, int H, const float* __restrict__ dcat,
                          const int* __restrict__ nbr, const float* __restrict__ g,
                          float* __restrict__ dh) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (size_t)n * H) return;
  const int i = (int)(q / H), c = (int)(q % H);
  const int s = i / n_per, k = i % n_per;
  const float* d = dcat + (size_t)i * 3 * H;
  float v = d[c];
  if (k > 0) v += dcat[(size_t)(i - 1) * 3 * H + H + c];
  if (k + 1 < n_per) v += dcat[(size_t)(i + 1) * 3 * H + H + c];
  atomicAdd(&dh[q], v);
  const float dn = d[2 * H + c];
#pragma unroll
  for (int m = 0; m < NB_K; ++m) {
    const float gm = g[s * NB_K + m];
    if (gm != 0.f) atomicAdd(&dh[((size_t)nbr[s * NB_K + m] * n_per + k) * H + c], gm * dn);
  }
}

// dZ = dh * (Z > 0).
__global__ void k_relu_bwd(size_t len, const float* __restrict__ dh, const float* __restrict__ Z,
                           float* __restrict__ dZ) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < len) dZ[i] = Z[i] > 0.f ? dh[i] : 0.f;
}

// ---- head, outputs and losses -------------------------------------------------------

// The Jacobi factor 1 / sqrt(1 + w^2 var_s) of a W-form pixel.
__device__ __forceinline__ float jacobi_factor(double w, double var_s) {
  return (float)(1.0 / sqrt(1.0 + w * w * var_s));
}

// y0 and the band rows of L from Y (n x NO, NO = 2 + B).
__global__ void k_outputs(int n, int n_per, int B, double var_s, const double* __restrict__ rec,
                          const float* __restrict__ Y, double* __restrict__ y0,
                          float* __restrict__ Lr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int NO = 2 + B, k = i % n_per;
  const float* y = Y + (size_t)i * NO;
  if (y0) y0[i] = (double)(XS * y[0]);
  float* l = Lr + (size_t)i * (B + 1);
  const float d = jacobi_factor(rec[(size_t)i * 5 + 3], var_s) * expf(SD * tanhf(y[1]));
  const float a2 = AC * tanhf(y[3]), a1 = AC * (1.f + a2) * tanhf(y[2]);
  l[0] = d;
  l[1] = k >= 1 ? a1 * d : 0.f;
  l[2] = k >= 2 ? a2 * d : 0.f;
}

// Warm-start loss sum (y0 - y*)^2 / sum y*^2: per-block partials of both
// sums (2 per block).
__global__ void k_xloss_part(int n, const float* __restrict__ Y, int NO,
                             const double* __restrict__ ystar, double* __restrict__ part) {
  __shared__ double red[2][8];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double e2 = 0.0, t2 = 0.0;
  if (i < n) {
    const double d = (double)(XS * Y[(size_t)i * NO]) - ystar[i];
    e2 = d * d;
    t2 = ystar[i] * ystar[i];
  }
  for (int o = 16; o > 0; o >>= 1) {
    e2 += __shfl_down_sync(0xffffffffu, e2, o);
    t2 += __shfl_down_sync(0xffffffffu, t2, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = e2;
    red[1][threadIdx.x >> 5] = t2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      a += red[0][w];
      b += red[1][w];
    }
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = b;
  }
}

// dY_0 of the warm-start loss (weight wx, normaliser sum y*^2 in *tot).
__global__ void k_xloss_grad(int n, const float* __restrict__ Y, int NO,
                             const double* __restrict__ ystar, const double* __restrict__ tot,
                             float wx, float* __restrict__ dY) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double d = (double)(XS * Y[(size_t)i * NO]) - ystar[i];
  dY[(size_t)i * NO] = (float)(wx * 2.0 * d * XS / tot[1]);
}

// Preconditioner loss of one skewer per CTA (n_per threads, n_per <= 1024):
// u = A_bb v, t = L^T u, s = L t, rho = s - v; loss sum rho^2 / n_total;
// dY_{1..1+B} of its pixels.
__global__ void k_ploss(int n_per, int B, int n_total, double var_s, double c_para,
                        const double* __restrict__ rec, const float* __restrict__ Y,
                        const float* __restrict__ probe, float wp, float* __restrict__ dY,
                        double* __restrict__ loss_part) {
  extern __shared__ float sm[];
  float* zz = sm;               // z
  float* ww = zz + n_per;       // w
  float* vv = ww + n_per;       // probe v
  float* uu = vv + n_per;       // A v
  float* tt = uu + n_per;       // L^T u
  float* gs = tt + n_per;       // d loss / d s
  float* L = gs + n_per;        // n_per x (B + 1) band rows
  const int s = blockIdx.x, k = threadIdx.x;
  const int i = s * n_per + k;
  const int NO = 2 + B;
  zz[k] = (float)rec[(size_t)i * 5 + 2];
  ww[k] = (float)rec[(size_t)i * 5 + 3];
  vv[k] = probe[i];
  const float* y = Y + (size_t)i * NO;
  const float dk = jacobi_factor(rec[(size_t)i * 5 + 3], var_s) * expf(SD * tanhf(y[1]));
  const float th2 = tanhf(y[2]), th3 = tanhf(y[3]);
  const float a2 = AC * th3, a1 = AC * (1.f + a2) * th2;
  L[k * (B + 1)] = dk;
  L[k * (B + 1) + 1] = k >= 1 ? a1 * dk : 0.f;
  L[k * (B + 1) + 2] = k >= 2 ? a2 * dk : 0.f;
  __syncthreads();
  // u = v + w S_bb w v  (the skewer's own block, exact kernel in FP32)
  float acc = 0.f;
  for (int j = 0; j < n_per; ++j) {
    const float dz = zz[k] - zz[j];
    acc = fmaf(__expf(-(float)c_para * dz * dz), ww[j] * vv[j], acc);
  }
  uu[k] = vv[k] + ww[k] * (float)var_s * acc;
  __syncthreads();
  // t_k = sum_m L[k+m][m] u_{k+m}
  float t = 0.f;
  for (int m = 0; m <= B; ++m)
    if (k + m < n_per) t = fmaf(L[(k + m) * (B + 1) + m], uu[k + m], t);
  tt[k] = t;
  __syncthreads();
  float sk = 0.f;
  for (int m = 0; m <= B; ++m)
    if (k - m >= 0) sk = fmaf(L[k * (B + 1) + m], tt[k - m], sk);
  const float rho = sk - vv[k];
  gs[k] = 2.f * wp * rho / n_total;
  __syncthreads();
  // g_t = L^T g_s; dL[k][m] = g_s[k] t[k-m] + g_t[k-m] u[k]
  float gt = 0.f;
  for (int m = 0; m <= B; ++m)
    if (k + m < n_per) gt = fmaf(L[(k + m) * (B + 1) + m], gs[k + m], gt);
  __syncthreads();
  tt[k] = gt;  // reuse: g_t (t itself kept in registers of its owner)
  __syncthreads();
  // this thread's t value again for the dL of rows k' = k + m is needed by
  // other threads: recompute locally from u (cheap) instead of sharing
  // d loss / d L[k][k-m] for the row's entries
  float dl[3] = {0.f, 0.f, 0.f};
  for (int m = 0; m <= B; ++m) {
    if (k - m < 0) continue;
    const int j = k - m;
    float tj = 0.f;  // t_j = sum_m' L[j+m'][m'] u_{j+m'}
    for (int mm = 0; mm <= B; ++mm)
      if (j + mm < n_per) tj = fmaf(L[(j + mm) * (B + 1) + mm], uu[j + mm], tj);
    dl[m] = gs[k] * tj + tt[j] * uu[k];
  }
  // chain rule through L_kk = J_k exp(SD tanh(Y1)), L_{k,k-1} = a1 L_kk,
  // L_{k,k-2} = a2 L_kk, a2 = AC tanh(Y3), a1 = AC (1 + a2) tanh(Y2)
  float* dy = dY + (size_t)i * NO;
  const float th1 = tanhf(y[1]);
  const float dkk = dl[0] + dl[1] * a1 + dl[2] * a2;  // through the diagonal
  dy[1] = dkk * dk * SD * (1.f - th1 * th1);
  dy[2] = dl[1] * AC * (1.f + a2) * (1.f - th2 * th2) * dk;
  dy[3] = (dl[1] * AC * th2 + dl[2]) * AC * (1.f - th3 * th3) * dk;
  // loss (n_per need not be a multiple of 32: a shared-memory sum in order)
  __syncthreads();
  uu[k] = rho * rho;
  __syncthreads();
  if (k == 0) {
    double a = 0.0;
    for (int j = 0; j < n_per; ++j) a += (double)uu[j];
    loss_part[s] = wp * a / n_total;
  }
}

// ---- optimiser ---------------------------------------------------------------------

__global__ void k_adam(size_t n, float lr, float b1, float b2, float eps, float bc1, float bc2,
                       float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

__global__ void k_to_bf16(size_t n, const float* __restrict__ p, __nv_bfloat16* __restrict__ q) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) q[i] = __float2bfloat16_rn(p[i]);
}

// Deterministic initial weights (uniform +-sqrt(3 / fan_in) from a hash).
__global__ void k_init(size_t n, unsigned seed, const int* __restrict__ fan_in_of,
                       const unsigned char* __restrict__ is_bias, float* __restrict__ p) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned x = (unsigned)i * 2654435761u ^ (seed * 2246822519u + 0x9e3779b9u);
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  const float u = (x >> 8) * (1.f / 16777216.f) * 2.f - 1.f;
  p[i] = is_bias[i] ? 0.f : u * sqrtf(3.f / fan_in_of[i]);
}

}  // namespace

// ---- host side ---------------------------------------------------------------------------

LearnedNet::LearnedNet(ds_context* c, int hidden, int band, const KernelConsts& k, unsigned seed)
    : ctx(c), H(hidden), B(band), kc(k) {
  require(H >= 32 && H % 32 == 0 && H <= 512, "hidden width must be a multiple of 32 in [32, 512]");
  require(B == 2, "the learned factor has band 2 (stability-triangle coefficients)");
  NO = 2 + B;
  // layout of the flat parameter vector
  auto add = [&](size_t rows, size_t cols, bool bias) {
    Slot sl{n_params, rows, cols, bias};
    n_params += rows * cols;
    return sl;
  };
  W_in = add(F_IN, H, false);
  b_in = add(1, H, true);
  for (int l = 0; l < N_LAYERS; ++l) {
    W_l[l] = add(3 * (size_t)H, H, false);
    b_l[l] = add(1, H, true);
  }
  W_o = add(H, NO, false);
  b_o = add(1, NO, true);
  params.alloc(n_params);
  grads.alloc(n_params);
  adam_m.alloc(n_params);
  adam_v.alloc(n_params);
  wbf.alloc(n_params);
  cudaStream_t st = ctx->stream;
  std::vector<int> fan(n_params);
  std::vector<unsigned char> isb(n_params, 0);
  auto mark = [&](const Slot& sl, int f) {
    for (size_t q = 0; q < sl.rows * sl.cols; ++q) {
      fan[sl.off + q] = f;
      isb[sl.off + q] = sl.bias ? 1 : 0;
    }
  };
  mark(W_in, F_IN);
  mark(b_in, 1);
  for (int l = 0; l < N_LAYERS; ++l) {
    mark(W_l[l], 3 * H);
    mark(b_l[l], 1);
  }
  mark(W_o, H);
  mark(b_o, 1);
  DevBuf<int> dfan;
  DevBuf<unsigned char> disb;
  dfan.alloc(n_params);
  disb.alloc(n_params);
  DS_CUDA(cudaMemcpyAsync(dfan.p, fan.data(), n_params * sizeof(int), cudaMemcpyHostToDevice, st));
  DS_CUDA(cudaMemcpyAsync(disb.p, isb.data(), n_params, cudaMemcpyHostToDevice, st));
  k_init<<<grid1(n_params), 256, 0, st>>>(n_params, seed, dfan.p, disb.p, params.p);
  DS_CHECK_LAUNCH();
  // The head starts at zero: y0 = 0 and L = the Jacobi factor (Y = 0), so
  // that the untrained network is Jacobi-PCG and training only improves it.
  DS_CUDA(cudaMemsetAsync(params.p + W_o.off, 0, (W_o.rows * W_o.cols + NO) * sizeof(float), st));
  DS_CUDA(cudaMemsetAsync(adam_m.p, 0, n_params * sizeof(float), st));
  DS_CUDA(cudaMemsetAsync(adam_v.p, 0, n_params * sizeof(float), st));
  sync_weights();
  DS_CUDA(cudaStreamSynchronize(st));
}

void LearnedNet::sync_weights() {
  k_to_bf16<<<grid1(n_params), 256, 0, ctx->stream>>>(
      n_params, params.p, reinterpret_cast<__nv_bfloat16*>(wbf.p));
  DS_CHECK_LAUNCH();
}

void LearnedNet::ensure(int n_sk, int n_per) {
  require(n_sk >= 1 && n_per >= 1 && n_per <= 1024, "n_per must be in [1, 1024]");
  const size_t n = (size_t)n_sk * n_per;
  if (n == n_cur && n_sk == nsk_cur) return;
  n_cur = n;
  nsk_cur = n_sk;
  nbr.alloc((size_t)n_sk * NB_K);
  gw.alloc((size_t)n_sk * NB_K);
  skxy.alloc(n_sk);
  X.alloc(n * F_IN);
  for (int l = 0; l <= N_LAYERS; ++l) {
    h[l].alloc(n * H);
    Z[l].alloc(n * H);
  }
  for (int l = 0; l < N_LAYERS; ++l) cat[l].alloc(n * 3 * H);
  Y.alloc(n * NO);
  dY.alloc(n * NO);
  dh.alloc(n * H);
  dh2.alloc(n * H);
  dZ.alloc(n * H);
  dcat.alloc(n * 3 * H);
  const size_t chunks = (n + ATB_CHUNK - 1) / ATB_CHUNK;
  part.alloc(chunks * std::max<size_t>(3 * (size_t)H * H, (size_t)H * NO));
  dpart.alloc(std::max<size_t>(2 * grid1(n), (size_t)n_sk) + 2);
}

void LearnedNet::gemm_fwd(int M, int N, int K, const float* A, int lda, const Slot& W, const Slot& b,
                          float* Zp, float* out, const float* res, int epi) {
  const dim3 grid((N + 63) / 64, (M + 63) / 64);
  const __nv_bfloat16* Wp = reinterpret_cast<const __nv_bfloat16*>(wbf.p) + W.off;
  const float* bp = params.p + b.off;
  cudaStream_t st = ctx->stream;
  if (epi == 0)
    k_gemm<false, 0><<<grid, 256, 0, st>>>(M, N, K, A, lda, Wp, N, bp, Zp, out, res, N);
  else if (epi == 1)
    k_gemm<false, 1><<<grid, 256, 0, st>>>(M, N, K, A, lda, Wp, N, bp, Zp, out, res, N);
  else
    k_gemm<false, 2><<<grid, 256, 0, st>>>(M, N, K, A, lda, Wp, N, bp, Zp, out, res, N);
  DS_CHECK_LAUNCH();
}

// dW (slot) = A^T D over M rows; db = column sums of D.
void LearnedNet::grad_w(int M, int K, int N, const float* A, int lda, const float* D,
                        const Slot& W, const Slot& b) {
  cudaStream_t st = ctx->stream;
  const int chunks = (M + ATB_CHUNK - 1) / ATB_CHUNK;
  const dim3 grid((N + 63) / 64, (K + 63) / 64, chunks);
  k_gemm_atb<<<grid, 256, 0, st>>>(M, K, N, A, lda, D, N, part.p);
  DS_CHECK_LAUNCH();
  k_reduce_chunks<<<grid1((size_t)K * N), 256, 0, st>>>(chunks, (size_t)K * N, part.p,
                                                        grads.p + W.off);
  DS_CHECK_LAUNCH();
  k_colsum_part<<<dim3(grid1(N, 128), chunks), 128, 0, st>>>(M, N, D, part.p);
  DS_CHECK_LAUNCH();
  k_reduce_chunks<<<grid1(N), 256, 0, st>>>(chunks, (size_t)N, part.p, grads.p + b.off);
  DS_CHECK_LAUNCH();
}

void LearnedNet::forward(int n_sk, int n_per, const double* rec) {
  ensure(n_sk, n_per);
  rec_cur = rec;
  cudaStream_t st = ctx->stream;
  const int n = n_sk * n_per;
  k_skewer_xy<<<grid1(n_sk), 256, 0, st>>>(n_sk, n_per, rec, skxy.p);
  DS_CHECK_LAUNCH();
  k_knn<<<grid1((size_t)n_sk * 32), 256, 0, st>>>(n_sk, skxy.p, kc.c_perp, nbr.p, gw.p);
  DS_CHECK_LAUNCH();
  k_features<<<grid1(n), 256, 0, st>>>(n, n_per, rec, gw.p, X.p);
  DS_CHECK_LAUNCH();
  gemm_fwd(n, H, F_IN, X.p, F_IN, W_in, b_in, Z[0].p, h[0].p, nullptr, 1);
  for (int l = 0; l < N_LAYERS; ++l) {
    k_agg_fwd<<<grid1((size_t)n * (H / 4)), 256, 0, st>>>(n, n_per, H, h[l].p, nbr.p, gw.p,
                                                          cat[l].p);
    DS_CHECK_LAUNCH();
    if (tc_active && layer_tc_usable(n, H, 3 * H)) {
      if (!wt.p) wt.alloc((size_t)3 * H * H);
      if (!tc_err.p) {
        tc_err.alloc(1);
        DS_CUDA(cudaMemsetAsync(tc_err.p, 0, sizeof(int), st));
      }
      // inference only: no Z (the backward pass alone reads it)
      launch_layer_tc(n, cat[l].p, reinterpret_cast<const __nv_bfloat16*>(wbf.p) + W_l[l].off,
                      params.p + b_l[l].off, nullptr, h[l + 1].p, h[l].p, wt.p, tc_err.p, st);
    } else {
      gemm_fwd(n, H, 3 * H, cat[l].p, 3 * H, W_l[l], b_l[l], Z[l + 1].p, h[l + 1].p, h[l].p, 2);
    }
  }
  gemm_fwd(n, NO, H, h[N_LAYERS].p, H, W_o, b_o, nullptr, Y.p, nullptr, 0);
}

void LearnedNet::outputs(int n_sk, int n_per, double* y0, float* Lrows) {
  const int n = n_sk * n_per;
  k_outputs<<<grid1(n), 256, 0, ctx->stream>>>(n, n_per, B, kc.var_s, rec_cur, Y.p, y0, Lrows);
  DS_CHECK_LAUNCH();
}

void LearnedNet::loss_and_grad(int n_sk, int n_per, const double* rec, const double* ystar,
                               const float* probe, float wx, float wp, double* losses) {
  cudaStream_t st = ctx->stream;
  const int n = n_sk * n_per;
  forward(n_sk, n_per, rec);
  DS_CUDA(cudaMemsetAsync(dY.p, 0, (size_t)n * NO * sizeof(float), st));
  // warm-start loss
  const unsigned gb = grid1(n);
  k_xloss_part<<<gb, 256, 0, st>>>(n, Y.p, NO, ystar, dpart.p);
  DS_CHECK_LAUNCH();
  std::vector<double> hp(2 * (size_t)gb);
  DS_CUDA(cudaMemcpyAsync(hp.data(), dpart.p, hp.size() * sizeof(double), cudaMemcpyDeviceToHost,
                          st));
  DS_CUDA(cudaStreamSynchronize(st));
  double e2 = 0.0, t2 = 0.0;
  for (unsigned b = 0; b < gb; ++b) {
    e2 += hp[2 * b];
    t2 += hp[2 * b + 1];
  }
  require(t2 > 0.0, "the target solution is zero");
  const double tot[2] = {e2, t2};
  DS_CUDA(cudaMemcpyAsync(dpart.p, tot, sizeof(tot), cudaMemcpyHostToDevice, st));
  k_xloss_grad<<<gb, 256, 0, st>>>(n, Y.p, NO, ystar, dpart.p, wx, dY.p);
  DS_CHECK_LAUNCH();
  DS_CUDA(cudaStreamSynchronize(st));  // tot is on this stack frame
  // preconditioner loss
  const size_t shm = (size_t)n_per * (6 + B + 1) * sizeof(float);
  k_ploss<<<n_sk, n_per, shm, st>>>(n_per, B, n, kc.var_s, kc.c_para, rec, Y.p, probe, wp, dY.p,
                                     dpart.p);
  DS_CHECK_LAUNCH();
  std::vector<double> lp(n_sk);
  DS_CUDA(cudaMemcpyAsync(lp.data(), dpart.p, n_sk * sizeof(double), cudaMemcpyDeviceToHost, st));
  DS_CUDA(cudaStreamSynchronize(st));
  double pl = 0.0;
  for (double v : lp) pl += v;
  losses[0] = wx * e2 / t2;
  losses[1] = pl;
  backward(n_sk, n_per);
}

void LearnedNet::backward(int n_sk, int n_per) {
  cudaStream_t st = ctx->stream;
  const int n = n_sk * n_per;
  // head: dW_o = h4^T dY, dh4 = dY W_o^T
  grad_w(n, H, NO, h[N_LAYERS].p, H, dY.p, W_o, b_o);
  {
    const dim3 grid((H + 63) / 64, (n + 63) / 64);
    const __nv_bfloat16* Wp = reinterpret_cast<const __nv_bfloat16*>(wbf.p) + W_o.off;
    k_gemm<true, 0><<<grid, 256, 0, st>>>(n, H, NO, dY.p, NO, Wp, NO, nullptr, nullptr, dh.p,
                                          nullptr, H);
    DS_CHECK_LAUNCH();
  }
  for (int l = N_LAYERS - 1; l >= 0; --l) {
    // h_{l+1} = h_l + relu(Z_{l+1}), Z_{l+1} = cat_l W_l + b_l
    k_relu_bwd<<<grid1((size_t)n * H), 256, 0, st>>>((size_t)n * H, dh.p, Z[l + 1].p, dZ.p);
    DS_CHECK_LAUNCH();
    grad_w(n, 3 * H, H, cat[l].p, 3 * H, dZ.p, W_l[l], b_l[l]);
    const dim3 grid((3 * H + 63) / 64, (n + 63) / 64);
    const __nv_bfloat16* Wp = reinterpret_cast<const __nv_bfloat16*>(wbf.p) + W_l[l].off;
    k_gemm<true, 0><<<grid, 256, 0, st>>>(n, 3 * H, H, dZ.p, H, Wp, H, nullptr, nullptr, dcat.p,
                                          nullptr, 3 * H);
    DS_CHECK_LAUNCH();
    // dh_l = dh_{l+1} (residual) + aggregation adjoint of dcat
    DS_CUDA(cudaMemcpyAsync(dh2.p, dh.p, (size_t)n * H * sizeof(float), cudaMemcpyDeviceToDevice,
                            st));
    k_agg_bwd<<<grid1((size_t)n * H), 256, 0, st>>>(n, n_per, H, dcat.p, nbr.p, gw.p, dh2.p);
    DS_CHECK_LAUNCH();
    std::swap(dh, dh2);
  }
  // embed: h0 = relu(Z0)
  k_relu_bwd<<<grid1((size_t)n * H), 256, 0, st>>>((size_t)n * H, dh.p, Z[0].p, dZ.p);
  DS_CHECK_LAUNCH();
  grad_w(n, F_IN, H, X.p, F_IN, dZ.p, W_in, b_in);
}

void LearnedNet::adam_step(float lr) {
  ++step;
  const float b1 = 0.9f, b2 = 0.999f;
  const float bc1 = 1.f - std::pow(b1, (float)step), bc2 = 1.f - std::pow(b2, (float)step);
  k_adam<<<grid1(n_params), 256, 0, ctx->stream>>>(n_params, lr, b1, b2, 1e-8f, bc1, bc2,
                                                   params.p, grads.p, adam_m.p, adam_v.p);
  DS_CHECK_LAUNCH();
  sync_weights();
}

void SkewerPCDeleter::operator()(SkewerPC* p) const { delete p; }

// Band rows [record][w] to planes [w][record] (the layout of SkewerPC::L).
__global__ void k_band_planes(size_t n, int w, const float* __restrict__ rows,
                              float* __restrict__ planes) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * w) return;
  planes[(i % w) * n + i / w] = rows[i];
}

}  // namespace ds

using namespace ds;

namespace {

constexpr char MAGIC[4] = {'D', 'S', 'L', 'N'};
constexpr int FILE_VERSION = 1;

}  // namespace

extern "C" {

int ds_operator_set_skewer_preconditioner(ds_operator* op, int n_skewers, int n_per, int band,
                                          const float* L_rows) {
  if (!op) return DS_ERR_ARG;
  return guarded(op->ctx, [&] {
    if (!L_rows) {
      op->pc.reset();
      return;
    }
    require(n_skewers > 0 && n_per > 0 && n_per <= 1024 && (long long)n_skewers * n_per == op->n,
            "n_skewers x n_per must equal the operator's record count (n_per <= 1024)");
    require(band >= 0 && band < n_per && band <= 32, "band must be in [0, min(n_per, 33))");
    std::unique_ptr<SkewerPC, SkewerPCDeleter> pc(new SkewerPC());
    pc->n_sk = n_skewers;
    pc->n_per = n_per;
    pc->band = band;
    pc->L.alloc((size_t)op->n * (band + 1));
    DevBuf<float> rows;  // the caller's rows, then their planes
    rows.alloc(pc->L.n);
    DS_CUDA(cudaMemcpyAsync(rows.p, L_rows, rows.bytes(), cudaMemcpyDefault, op->ctx->stream));
    k_band_planes<<<(unsigned)((rows.n + 255) / 256), 256, 0, op->ctx->stream>>>(
        (size_t)op->n, band + 1, rows.p, pc->L.p);
    DS_CHECK_LAUNCH();
    DS_CUDA(cudaStreamSynchronize(op->ctx->stream));
    op->pc = std::move(pc);
  });
}

int ds_learned_create(ds_context* ctx, const ds_kernel_params* kp, int hidden, int band,
                      unsigned seed, ds_learned** out) {
  if (!ctx || !kp || !out) return DS_ERR_ARG;
  *out = nullptr;
  auto h = std::make_unique<ds_learned>();
  const int rc = guarded(ctx, [&] {
    require(kp->eval == DS_EVAL_EXACT, "the learned preconditioner uses the exact kernel");
    DS_CUDA(cudaSetDevice(ctx->device));
    h->net.reset(new LearnedNet(ctx, hidden, band, make_consts(*kp), seed));
  });
  if (rc != DS_OK) return rc;
  *out = h.release();
  return DS_OK;
}

void ds_learned_destroy(ds_learned* h) { delete h; }

int ds_learned_num_params(ds_learned* h, long long* n) {
  if (!h || !n) return DS_ERR_ARG;
  *n = (long long)h->net->n_params;
  return DS_OK;
}

static int learned_copy(ds_learned* h, float* dst, const float* src, bool to_host,
                        bool sync_after) {
  if (!h || !(to_host ? dst : src)) return DS_ERR_ARG;
  LearnedNet& net = *h->net;
  return guarded(net.ctx, [&] {
    cudaStream_t st = net.ctx->stream;
    const size_t bytes = net.n_params * sizeof(float);
    if (to_host) {
      DS_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st));
    } else {
      DS_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
      if (sync_after) net.sync_weights();
    }
    DS_CUDA(cudaStreamSynchronize(st));
  });
}

int ds_learned_get_params(ds_learned* h, float* params) {
  return h ? learned_copy(h, params, h->net->params.p, true, false) : DS_ERR_ARG;
}

int ds_learned_set_params(ds_learned* h, const float* params) {
  return h ? learned_copy(h, h->net->params.p, params, false, true) : DS_ERR_ARG;
}

int ds_learned_get_grads(ds_learned* h, float* grads) {
  return h ? learned_copy(h, grads, h->net->grads.p, true, false) : DS_ERR_ARG;
}

int ds_learned_save(ds_learned* h, const char* path) {
  if (!h || !path) return DS_ERR_ARG;
  LearnedNet& net = *h->net;
  return guarded(net.ctx, [&] {
    std::vector<float> p(net.n_params);
    DS_CUDA(cudaMemcpyAsync(p.data(), net.params.p, p.size() * sizeof(float), cudaMemcpyDeviceToHost, net.ctx->stream));
    DS_CUDA(cudaStreamSynchronize(net.ctx->stream));
    FILE* f = fopen(path, "wb");
    require(f != nullptr, "cannot open the weight file for writing");
    const int hdr[3] = {FILE_VERSION, net.H, net.B};
    const long long np = (long long)net.n_params;
    const bool ok = fwrite(MAGIC, 1, 4, f) == 4 && fwrite(hdr, sizeof(int), 3, f) == 3 &&
                    fwrite(&np, sizeof(np), 1, f) == 1 &&
                    fwrite(p.data(), sizeof(float), p.size(), f) == p.size();
    fclose(f);
    require(ok, "writing the weight file failed");
  });
}

int ds_learned_load(ds_learned* h, const char* path) {
  if (!h || !path) return DS_ERR_ARG;
  LearnedNet& net = *h->net;
  return guarded(net.ctx, [&] {
    FILE* f = fopen(path, "rb");
    require(f != nullptr, "cannot open the weight file");
    char magic[4] = {0, 0, 0, 0};
    int hdr[3] = {0, 0, 0};
    long long np = 0;
    std::vector<float> p(net.n_params);
    const bool ok = fread(magic, 1, 4, f) == 4 && std::memcmp(magic, MAGIC, 4) == 0 &&
                    fread(hdr, sizeof(int), 3, f) == 3 && hdr[0] == FILE_VERSION &&
                    hdr[1] == net.H && hdr[2] == net.B && fread(&np, sizeof(np), 1, f) == 1 &&
                    np == (long long)net.n_params &&
                    fread(p.data(), sizeof(float), p.size(), f) == p.size();
    fclose(f);
    require(ok, "the weight file does not match this network (format, width or band)");
    DS_CUDA(cudaMemcpyAsync(net.params.p, p.data(), p.size() * sizeof(float), cudaMemcpyHostToDevice, net.ctx->stream));
    DS_CUDA(cudaStreamSynchronize(net.ctx->stream));
    net.sync_weights();
    DS_CUDA(cudaStreamSynchronize(net.ctx->stream));
  });
}

int ds_learned_forward_dev(ds_learned* h, int n_skewers, int n_per, const double* records,
                           double* y0, float* L_rows) {
  if (!h || !records || !L_rows) return DS_ERR_ARG;
  LearnedNet& net = *h->net;
  return guarded(net.ctx, [&] {
    net.tc_active = net.tc_infer;
    try {
      net.forward(n_skewers, n_per, records);
    } catch (...) {
      net.tc_active = false;
      throw;
    }
    net.tc_active = false;
    net.outputs(n_skewers, n_per, y0, L_rows);
    if (net.tc_err.p) {
      int code = 0;
      DS_CUDA(cudaMemcpyAsync(&code, net.tc_err.p, sizeof(int), cudaMemcpyDeviceToHost, net.ctx->stream));
      DS_CUDA(cudaStreamSynchronize(net.ctx->stream));
      if (code) {
        DS_CUDA(cudaMemsetAsync(net.tc_err.p, 0, sizeof(int), net.ctx->stream));
        throw Error{DS_ERR_CUDA, "tensor-core layer GEMM: an mbarrier wait timed out (code " +
                                     std::to_string(code) + ")"};
      }
    }
  });
}

int ds_learned_set_inference(ds_learned* h, int tensor_cores) {
  if (!h) return DS_ERR_ARG;
  h->net->tc_infer = tensor_cores != 0;
  return DS_OK;
}

int ds_learned_train_step_dev(ds_learned* h, int n_skewers, int n_per, const double* records,
                              const double* y_star, const float* probe, float lr, float w_x,
                              float w_p, int update, double* losses) {
  if (!h || !records || !y_star || !probe || !losses) return DS_ERR_ARG;
  LearnedNet& net = *h->net;
  return guarded(net.ctx, [&] {
    net.loss_and_grad(n_skewers, n_per, records, y_star, probe, w_x, w_p, losses);
    if (update) net.adam_step(lr);
  });
}

}  // extern "C"
