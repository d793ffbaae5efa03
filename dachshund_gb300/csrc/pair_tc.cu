// FP32 inner matvec q = A32 p of the mixed-precision form with the pair
// exponents on the tensor cores.
//
// The EXPANDED exponent of a (row i, column j) pair, in log2 units, with xi
// the coordinates relative to each point's tile origin and d = o_C - o_R the
// offset of the column tile's origin from the row tile's, is
//   t_ij = 2 xi_i . (xi_j + d) - |xi_j + d|^2      (= |xi_i|^2 - |xi_i - xi_j - d|^2)
//        = 2 y_i . xi_j - |xi_j|^2 + r_i,  y_i = xi_i - d,  r_i = 2 xi_i . d - |d|^2,
// and the product term e_ij u_j (u_j = w_j p_j) is
//   e_ij u_j = sign(u_j) 2^(t_ij + log2 |u_j|).
// So per 128 x 128 tile pair tcgen05.mma (kind::tf32, M = N = 128) forms
// T_ij = t_ij + log2 |u_j| in tensor memory from a row operand (y_i, r_i, 1)
// rebuilt per tile pair and a column operand (2 xi_j, 1, c_j),
// c_j = log2 |u_j| - |xi_j|^2, that depends on the column tile only and is
// written for all columns once per product (k_tc_columns); a third MMA
// broadcasts sign(u_j) to every row (S_ij = sign(u_j)).  The consumer warps
// then spend per pair one MUFU ex2 and half a packed FMA:
// acc_i += 2^T_ij S_ij.  The CUDA-core kernel (pair_f32.cu) spends 4 FMA
// lanes and one ex2 per pair; here the FMA pipe is nearly idle and the kernel
// is bound by ex2 (32 per clock per SM).
//
// Precision (3xTF32): an FP32 operand x is split into x_hi (x with its low 13
// mantissa bits cleared, exact in TF32) and x_lo = round_tf32(x - x_hi); the
// products use x_hi y_hi + x_hi y_lo + x_lo y_hi (relative error about 2^-21
// per product term) and c_j, r_i are carried in three TF32 pieces (exact).
// The operand K slots (two MMAs of K = 8):
//   A1 = [y_hi 1 | y_hi r_hi]       B1 = [2xi_hi c_hi | 2xi_lo 1]
//   A2 = [y_lo 1 | 1 r_mid r_lo 0]  B2 = [2xi_hi c_mid | c_lo 1 1 s]
//   AS = [0 0 0 0 | 0 0 0 1]        T = A1 B1 + A2 B2,  S = AS B2
// (y, xi: 3 slots each).  The exponent error is about 2^-21 (|2 y . xi| +
// |xi|^2) plus the FP32 rounding of r_i, a relative error of e_ij near 1e-6
// for neighbouring tiles, larger only where e_ij is small: the inner
// operator of the mixed solver, whose FP64-accurate reliable updates remove
// it.
//
// Per CTA (one per SM, persistent over row tiles, items dealt round-robin in
// the heaviest-first order), warp-specialized with mbarrier hand-offs:
//   * warps 0-15 (consumers): warp w reads TMEM lanes 32 (w % 4) .. + 31 (its
//     rows) and column sub-tile w / 4 of each tile, skips it when it is
//     outside the cutoff, and folds each tile's sum into a Kahan-compensated
//     FP32 row sum; after a row tile the four column quarters are added in
//     FP64 and q = rowf sum + ediag p is written, with the fused p.q partial
//     of the CG step;
//   * warps 16-17 (producers) rebuild the row operand of each tile pair (64
//     rows each, from the row tile's coordinates held in registers; 4
//     stages);
//   * lane 0 of warp 18 copies the column operand of each tile pair
//     (cp.async.bulk, 8 KB) into its stage as soon as the stage is free;
//   * lane 0 of warp 19 issues the MMAs into one of two TMEM buffers (T and S,
//     256 of the 512 columns each) and commits them.
// Every mbarrier wait is bounded: on a time-out the kernel records an error
// code, waits (bounded) for its MMAs and copies in flight, frees its tensor
// memory and returns.
//
// Measured on GB300 (262,144-pixel workload): 0.36 ms per product against
// 0.22 ms for the CUDA-core kernel, with ex2 at 28% of its peak.  Per
// 128 x 128 tile the three TF32 MMAs take ~400 clocks to issue and each
// consumer warp ~900 clocks for its 32 x 32 sub-tile (TMEM-load latency not
// hidden: T and S fill all 512 TMEM columns with two buffers).  The kernel is
// therefore opt-in (DS_INNER_TENSOR); its parity with the CUDA-core kernel
// and the FP64 solve is tested.
#include "ds_device.cuh"
#include "ds_f32.h"
#include "ds_tc.cuh"

#include <algorithm>

namespace ds {
namespace {

constexpr int PT_CONS = 16;                     // consumer warps
constexpr int PT_PROD = 2;                      // producer warps
constexpr int PT_COPY = PT_CONS + PT_PROD;       // column-operand copier warp
constexpr int PT_MMA = PT_COPY + 1;               // MMA warp
constexpr int PT_THREADS = (PT_MMA + 1) * 32;
// one CTA per SM: registers of the busiest of the 4 SM sub-partitions
constexpr int PT_MAXNREG = (16384 / (32 * ((PT_THREADS / 32 + 3) / 4))) & ~7;
constexpr int PT_STAGES = 4;                    // column-operand stages
constexpr int OP_K = 8;                         // TF32 K per MMA (32 bytes per row)
constexpr int OP_ELEMS = TILE * OP_K;           // one 128-row K = 8 operand (4 KB)
constexpr uint32_t OP_LBO = (TILE / 8) * 128;   // K-adjacent core matrices
constexpr uint32_t OP_SBO = 128;                // 8-row groups
constexpr uint32_t PT_TMEM_COLS = 512;          // 2 buffers x (T 128 + S 128)
constexpr uint32_t PT_IDESC = idesc_tf32(TILE, TILE);

// Element (row r, k) of a 128-row, K = 8 operand in the canonical K-major
// no-swizzle layout (core matrices of 8 rows x 16 bytes, 4-byte elements).
__device__ __forceinline__ int op_at(int r, int k) {
  return ((k >> 2) * (TILE / 8) + (r >> 3)) * 32 + (r & 7) * 4 + (k & 3);
}

__device__ __forceinline__ float tf32_hi(float x) {
  return __uint_as_float(__float_as_uint(x) & 0xffffe000u);
}
__device__ __forceinline__ float tf32_rn(float x) {
  return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xffffe000u);
}

__device__ __forceinline__ float ex2_pt(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ float lg2_pt(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ void kahan_add_pt(float& s, float& c, float v) {
  const float y = v - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

struct PtSmem {
  float a[PT_STAGES][2][OP_ELEMS];   // [stage][A1, A2] row operands
  float b[PT_STAGES][2][OP_ELEMS];   // [stage][B1, B2] column operands (bulk copies)
  float as[OP_ELEMS];                // sign selector (constant)
  double red[2][4][TILE];            // [item buffer][column quarter][row] row sums
  uint64_t a_full[PT_STAGES];        // row operand built       (PT_PROD arrives)
  uint64_t b_full[PT_STAGES];        // column operand landed   (1 arrive + tx bytes)
  uint64_t s_empty[PT_STAGES];       // MMAs reading the stage done (tcgen05.commit)
  uint64_t t_full[2], t_empty[2];    // MMAs of a tile done / T, S read back
  uint64_t row_done[2];              // the four column quarters' row sums written
  uint64_t red_free[2];              // row sums of the buffer read (4 arrives)
  uint32_t tmem_addr;
  int abort;
};

// The dynamic allocation is padded past half of the SM's shared memory so
// that one CTA, owning all 512 TMEM columns, runs per SM.
constexpr size_t PT_SMEM_BYTES = 120 * 1024;
static_assert(sizeof(PtSmem) + 1024 <= PT_SMEM_BYTES, "shared-memory layout");

__device__ __forceinline__ bool pt_wait(PtSmem& sm, uint64_t* bar, uint32_t parity, int* err,
                                        int code) {
  if (mbar_wait(bar, parity)) return true;
  if (err) atomicExch(err, code);
  *(volatile int*)&sm.abort = 1;
  return false;
}

__device__ __forceinline__ bool pt_warp_wait(PtSmem& sm, uint64_t* bar, uint32_t parity, int* err,
                                             int code, int lane) {
  int ok = 1;
  if (lane == 0) ok = pt_wait(sm, bar, parity, err, code);
  ok = __shfl_sync(0xffffffffu, ok, 0);
  __syncwarp();
  return ok != 0;
}

__device__ __forceinline__ bool pt_aborted(const PtSmem& sm) {
  return *(const volatile int*)&sm.abort != 0;
}

// Column operands of all column tiles for the product with u = colw v: per
// tile the 8 KB block [B1 | B2] in the operand layout, so a tile pair copies
// its column operand with one bulk copy.  One thread per column.
__global__ void k_tc_columns(int n, const float4* __restrict__ xi, const float* __restrict__ colw,
                             const float* __restrict__ v, const int* skip_flag,
                             float* __restrict__ out) {
  if (skip_flag && *skip_flag) return;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const float4 x = xi[j];
  const float u = colw[j] * v[j];
  // log2|u| (a zero u gives a term 2^-200 that flushes to zero)
  const float l = u != 0.f ? fmaxf(lg2_pt(fabsf(u)), -200.f) : -200.f;
  const float nx = -fmaf(x.x, x.x, fmaf(x.y, x.y, x.z * x.z));
  // c = l - |xi|^2 as an unevaluated pair, then three TF32 pieces
  const float cs0 = l + nx;
  const float bb = cs0 - l;
  const float ce = (l - (cs0 - bb)) + (nx - bb);
  const float ch = tf32_hi(cs0);
  const float r1 = cs0 - ch;
  const float cm = tf32_hi(r1);
  const float cl = tf32_rn((r1 - cm) + ce);
  const float sx = 2.f * x.x, sy = 2.f * x.y, sz = 2.f * x.z;
  const float sxh = tf32_hi(sx), syh = tf32_hi(sy), szh = tf32_hi(sz);
  float* B1 = out + (size_t)(j / TILE) * (2 * OP_ELEMS);
  float* B2 = B1 + OP_ELEMS;
  const int r = j % TILE;
  *reinterpret_cast<float4*>(B1 + op_at(r, 0)) = make_float4(sxh, syh, szh, ch);
  *reinterpret_cast<float4*>(B1 + op_at(r, 4)) =
      make_float4(tf32_rn(sx - sxh), tf32_rn(sy - syh), tf32_rn(sz - szh), 1.f);
  *reinterpret_cast<float4*>(B2 + op_at(r, 0)) = make_float4(sxh, syh, szh, cm);
  *reinterpret_cast<float4*>(B2 + op_at(r, 4)) = make_float4(cl, 1.f, 1.f, u < 0.f ? -1.f : 1.f);
}

template <bool DOT>
__global__ void __maxnreg__(PT_MAXNREG) k_pair_tc(F32Args a) {
  if (a.skip_flag && *a.skip_flag) return;
  extern __shared__ uint8_t smem_raw[];
  PtSmem& sm = *reinterpret_cast<PtSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                          ~uintptr_t(1023));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int s = 0; s < PT_STAGES; ++s) {
      mbar_init(&sm.a_full[s], PT_PROD);
      mbar_init(&sm.b_full[s], 1);
      mbar_init(&sm.s_empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&sm.t_full[b], 1);
      mbar_init(&sm.t_empty[b], PT_CONS);
      mbar_init(&sm.row_done[b], PT_CONS);
      mbar_init(&sm.red_free[b], 4);
    }
    sm.abort = 0;
    mbar_fence_init();
  }
  // AS: a 1 in K slot 7 of every row (selects the sign slot of B2)
  for (int e = tid; e < OP_ELEMS; e += PT_THREADS)
    sm.as[e] = ((e & 3) == 3 && (e >> 9) == 1) ? 1.f : 0.f;
  fence_async_smem();
  if (warp == 0) tmem_alloc(&sm.tmem_addr, PT_TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = sm.tmem_addr;
  const int n_items = a.n_row_tiles;
  int last_g = -1;  // the MMA thread's last committed tile / the copier's last copy

  if (warp < PT_CONS) {
    // ---- consumers ----------------------------------------------------------
    const int rs = warp & 3, cs = warp >> 2;
    const int row = 32 * rs + lane;
    double dot = 0.0;
    unsigned long long n_sub = 0;
    uint32_t g = 0, kc = 0;
    for (int item = blockIdx.x; item < n_items; item += gridDim.x, ++kc) {
      const int t = a.row_order ? a.row_order[item] : item;
      const int p0 = a.row_ptr[t], p1 = a.row_ptr[t + 1];
      float s = 0.f, c = 0.f;
      unsigned m = p0 < p1 ? a.mask[p0] : 0u;
      bool ok = true;
      for (int p = p0; p < p1; ++p, ++g) {
        const uint32_t b = g & 1;
        const unsigned mnext = p + 1 < p1 ? a.mask[p + 1] : 0u;
        if (!pt_warp_wait(sm, &sm.t_full[b], (g >> 1) & 1u, a.err, 41, lane)) {
          ok = false;
          break;
        }
        tc_fence_after();
        if ((m >> (4 * rs + cs)) & 1u) {  // warp-uniform
          ++n_sub;
          const uint32_t ta = tmem + ((uint32_t)(32 * rs) << 16) + b * 256u + 32u * cs;
          float tv[32], sv[32];
          tmem_ld32x2(ta, ta + 128u, tv, sv);
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&sm.t_empty[b]);
          float2 acc0 = make_float2(0.f, 0.f), acc1 = make_float2(0.f, 0.f);
#pragma unroll
          for (int k = 0; k < 32; k += 4) {
            acc0 = __ffma2_rn(make_float2(ex2_pt(tv[k]), ex2_pt(tv[k + 1])),
                              make_float2(sv[k], sv[k + 1]), acc0);
            acc1 = __ffma2_rn(make_float2(ex2_pt(tv[k + 2]), ex2_pt(tv[k + 3])),
                              make_float2(sv[k + 2], sv[k + 3]), acc1);
          }
          kahan_add_pt(s, c, (acc0.x + acc0.y) + (acc1.x + acc1.y));
        } else {
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&sm.t_empty[b]);
        }
        m = mnext;
      }
      if (!ok) break;
      // row sums of the four column quarters, added in FP64 by the quarter-0
      // warps; buffer kb is rewritten once they have read it two items ago
      const uint32_t kb = kc & 1;
      if (kc >= 2 &&
          !pt_warp_wait(sm, &sm.red_free[kb], ((kc >> 1) - 1) & 1u, a.err, 43, lane))
        break;
      sm.red[kb][cs][row] = (double)s - (double)c;
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.row_done[kb]);
      if (cs == 0) {
        if (!pt_warp_wait(sm, &sm.row_done[kb], (kc >> 1) & 1u, a.err, 42, lane)) break;
        const double sum = (sm.red[kb][0][row] + sm.red[kb][1][row]) +
                           (sm.red[kb][2][row] + sm.red[kb][3][row]);
        __syncwarp();
        if (lane == 0) mbar_arrive(&sm.red_free[kb]);
        const int i = t * TILE + row;
        const float q = fmaf(a.rowf[i], (float)sum, a.ediag[i] * a.vrow[i]);
        a.out[i] = q;
        if (DOT) dot += (double)a.dotv[i] * (double)q;
      }
    }
    if (a.prof_pairs && lane == 0) atomicAdd(a.prof_pairs, n_sub * SUBTILE * SUBTILE);
    if (DOT && cs == 0 && !pt_aborted(sm)) {
      // p.q: one partial per (CTA, row sub-tile); the last of the 4 x grid
      // warps to arrive adds them in a fixed order
      for (int o = 16; o > 0; o >>= 1) dot += __shfl_down_sync(0xffffffffu, dot, o);
      unsigned last = 0;
      if (lane == 0) {
        a.dot_partial[blockIdx.x * 4 + rs] = dot;
        __threadfence();
        last = atomicAdd(a.counter, 1u) == 4u * gridDim.x - 1u;
      }
      last = __shfl_sync(0xffffffffu, last, 0);
      if (last) {
        __threadfence();
        double v = 0.0;
        for (int k = lane; k < 4 * (int)gridDim.x; k += 32) v += __ldcg(a.dot_partial + k);
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) {
          *a.den_out = v;
          *a.alpha_out = *a.num / v;
          *a.counter = 0;
        }
      }
    }
  } else if (warp < PT_CONS + PT_PROD) {
    // ---- producers ------------------------------------------------------------
    // Producer pw builds rows c0, c0 + 32 (c0 = lane + 64 pw) of the row
    // operand of every tile pair.  The inputs of the next row tile and the
    // column-tile origins of the next 32 tile pairs are loaded ahead (one tile
    // pair per lane, read by shuffles), so no global-memory latency is waited
    // for per tile pair.
    const int pw = warp - PT_CONS;
    const int c0 = lane + 64 * pw;
    struct ItemIn {
      int t, p0, p1;
      float4 ot, x0, x1;
      float4 co0, co1;  // origins of the column tiles of pairs p0 + lane, p0 + 32 + lane
    };
    auto load_item = [&](int item) {
      ItemIn it;
      it.t = a.row_order ? a.row_order[item] : item;
      it.p0 = a.row_ptr[it.t];
      it.p1 = a.row_ptr[it.t + 1];
      it.ot = a.rorig[it.t];
      it.x0 = a.rxi[it.t * TILE + c0];
      it.x1 = a.rxi[it.t * TILE + c0 + 32];
      it.co0 = a.corig[it.p0 + lane < it.p1 ? a.cols[it.p0 + lane] : 0];
      it.co1 = a.corig[it.p0 + 32 + lane < it.p1 ? a.cols[it.p0 + 32 + lane] : 0];
      return it;
    };
    uint32_t g = 0;
    bool ok = true;
    ItemIn cur;
    if (blockIdx.x < n_items) cur = load_item(blockIdx.x);
    for (int item = blockIdx.x; item < n_items && ok; item += gridDim.x) {
      ItemIn nxt = cur;
      if (item + (int)gridDim.x < n_items) nxt = load_item(item + gridDim.x);
      const int p0 = cur.p0, p1 = cur.p1;
      int base = p0;
      float4 co0 = cur.co0, co1 = cur.co1;
      for (int p = p0; p < p1; ++p, ++g) {
        const uint32_t st = g % PT_STAGES;
        if (p - base == 32) {
          base = p;
          co0 = co1;
          co1 = a.corig[base + 32 + lane < p1 ? a.cols[base + 32 + lane] : 0];
        }
        // the row operand of stage st is free once the MMAs of tile pair
        // g - PT_STAGES completed
        if (g >= PT_STAGES &&
            !pt_warp_wait(sm, &sm.s_empty[st], ((g / PT_STAGES) - 1) & 1u, a.err, 52, lane)) {
          ok = false;
          break;
        }
        const float cox = __shfl_sync(0xffffffffu, co0.x, p - base);
        const float coy = __shfl_sync(0xffffffffu, co0.y, p - base);
        const float coz = __shfl_sync(0xffffffffu, co0.z, p - base);
        const float dx = cox - cur.ot.x, dy = coy - cur.ot.y, dz = coz - cur.ot.z;
        const float dd = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        float* A1 = sm.a[st][0];
        float* A2 = sm.a[st][1];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const float4 x = q == 0 ? cur.x0 : cur.x1;
          const int r = c0 + 32 * q;
          const float yx = x.x - dx, yy = x.y - dy, yz = x.z - dz;
          const float rr = fmaf(2.f * x.x, dx, fmaf(2.f * x.y, dy, fmaf(2.f * x.z, dz, -dd)));
          const float yxh = tf32_hi(yx), yyh = tf32_hi(yy), yzh = tf32_hi(yz);
          const float rh = tf32_hi(rr);
          const float r1 = rr - rh;
          const float rm = tf32_hi(r1);
          const float rl = tf32_rn(r1 - rm);
          *reinterpret_cast<float4*>(A1 + op_at(r, 0)) = make_float4(yxh, yyh, yzh, 1.f);
          *reinterpret_cast<float4*>(A1 + op_at(r, 4)) = make_float4(yxh, yyh, yzh, rh);
          *reinterpret_cast<float4*>(A2 + op_at(r, 0)) =
              make_float4(tf32_rn(yx - yxh), tf32_rn(yy - yyh), tf32_rn(yz - yzh), 1.f);
          *reinterpret_cast<float4*>(A2 + op_at(r, 4)) = make_float4(1.f, rm, rl, 0.f);
        }
        fence_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(&sm.a_full[st]);
      }
      cur = nxt;
    }
  } else if (warp == PT_COPY) {
    // ---- copier: column operand of each tile pair into its stage ---------------
    // column tiles of the next 32 tile pairs are loaded ahead, one per lane
    uint32_t g = 0;
    bool ok = true;
    for (int item = blockIdx.x; item < n_items && ok; item += gridDim.x) {
      const int t = a.row_order ? a.row_order[item] : item;
      const int p0 = a.row_ptr[t], p1 = a.row_ptr[t + 1];
      int base = p0;
      int ct0 = p0 + lane < p1 ? a.cols[p0 + lane] : 0;
      int ct1 = p0 + 32 + lane < p1 ? a.cols[p0 + 32 + lane] : 0;
      for (int p = p0; p < p1; ++p, ++g) {
        if (p - base == 32) {
          base = p;
          ct0 = ct1;
          ct1 = base + 32 + lane < p1 ? a.cols[base + 32 + lane] : 0;
        }
        const int ct = __shfl_sync(0xffffffffu, ct0, p - base);
        const uint32_t st = g % PT_STAGES;
        int okq = 1;
        if (lane == 0) {
          if (g >= PT_STAGES &&
              !pt_wait(sm, &sm.s_empty[st], ((g / PT_STAGES) - 1) & 1u, a.err, 53)) {
            okq = 0;
          } else {
            mbar_expect_tx(&sm.b_full[st], 2 * OP_ELEMS * 4);
            bulk_g2s(sm.b[st], a.tc_cols + (size_t)ct * (2 * OP_ELEMS), 2 * OP_ELEMS * 4,
                     &sm.b_full[st]);
            last_g = (int)g;
          }
        }
        if (!__shfl_sync(0xffffffffu, okq, 0)) {
          ok = false;
          break;
        }
      }
    }
  } else if (lane == 0) {
    // ---- MMA issue (warp PT_MMA) ------------------------------------------------------------
    uint32_t g = 0;
    const uint64_t as = sdesc(smem_u32(sm.as), OP_LBO, OP_SBO);
    bool ok = true;
    for (int item = blockIdx.x; item < n_items && ok; item += gridDim.x) {
      const int t = a.row_order ? a.row_order[item] : item;
      const int p0 = a.row_ptr[t], p1 = a.row_ptr[t + 1];
      for (int p = p0; p < p1; ++p, ++g) {
        const uint32_t st = g % PT_STAGES, b = g & 1;
        if (!pt_wait(sm, &sm.b_full[st], (g / PT_STAGES) & 1u, a.err, 62) ||
            !pt_wait(sm, &sm.a_full[st], (g / PT_STAGES) & 1u, a.err, 61) ||
            (g >= 2 && !pt_wait(sm, &sm.t_empty[b], ((g >> 1) - 1) & 1u, a.err, 63))) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint64_t a1 = sdesc(smem_u32(sm.a[st][0]), OP_LBO, OP_SBO);
        const uint64_t a2 = sdesc(smem_u32(sm.a[st][1]), OP_LBO, OP_SBO);
        const uint64_t b1 = sdesc(smem_u32(sm.b[st][0]), OP_LBO, OP_SBO);
        const uint64_t b2 = sdesc(smem_u32(sm.b[st][1]), OP_LBO, OP_SBO);
        const uint32_t dt = tmem + b * 256u;
        mma_tf32(dt, a1, b1, PT_IDESC, 0u);
        mma_tf32(dt, a2, b2, PT_IDESC, 1u);
        mma_tf32(dt + 128u, as, b2, PT_IDESC, 0u);
        mma_commit(&sm.s_empty[st]);
        mma_commit(&sm.t_full[b]);
        last_g = (int)g;
      }
    }
  }
  // teardown: after a time-out the MMA thread waits (bounded) for its MMAs in
  // flight and the copier for its last copy before the memory is released
  if (pt_aborted(sm) && lane == 0 && last_g >= 0) {
    if (warp == PT_MMA) mbar_wait(&sm.t_full[last_g & 1], (last_g >> 1) & 1u);
    if (warp == PT_COPY) mbar_wait(&sm.b_full[last_g % PT_STAGES], (last_g / PT_STAGES) & 1u);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, PT_TMEM_COLS);
}

}  // namespace

bool pair_tc_usable(int formula, int epi, const F32Args& a) {
  return formula == F32_EXPANDED && epi == EPI_PRODUCT && a.err != nullptr &&
         a.tc_cols != nullptr;
}

void launch_pair_tc(const F32Args& a0, cudaStream_t st) {
  if (a0.n_row_tiles <= 0) return;
  F32Args a = a0;
  cudaEvent_t ev = nullptr;
  if (a.prof && a.prof->enabled) {
    a.prof_pairs = a.prof->d_pairs + 1;
    a.prof->begin(st, &ev);
  } else {
    a.prof_pairs = nullptr;
  }
  static bool attr = false;
  if (!attr) {
    DS_CUDA(cudaFuncSetAttribute(k_pair_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)PT_SMEM_BYTES));
    DS_CUDA(cudaFuncSetAttribute(k_pair_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)PT_SMEM_BYTES));
    attr = true;
  }
  static int sms = 0;  // queried on the first (uncaptured) launch
  if (!sms) {
    int dev = 0;
    DS_CUDA(cudaGetDevice(&dev));
    DS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  }
  const int n_cols = a.n_row_tiles * TILE;
  k_tc_columns<<<(n_cols + 255) / 256, 256, 0, st>>>(n_cols, a.cxi, a.colw, a.v, a.skip_flag,
                                                    a.tc_cols);
  DS_CHECK_LAUNCH();
  const int grid = std::max(1, std::min(a.n_row_tiles, sms));
  if (a.dot_partial)
    k_pair_tc<true><<<grid, PT_THREADS, PT_SMEM_BYTES, st>>>(a);
  else
    k_pair_tc<false><<<grid, PT_THREADS, PT_SMEM_BYTES, st>>>(a);
  DS_CHECK_LAUNCH();
  if (ev) a.prof->end(st, ev, 1);
}

}  // namespace ds
