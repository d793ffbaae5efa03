// Multi-RHS matvec of the batched solver on the 5th-generation tensor cores:
// each generated S tile (128 rows x 128 columns of one tile pair) times the
// block of NB right-hand sides of the column tile is a BF16 contraction with
// FP32 accumulation in tensor memory (tcgen05.mma, kind::f16, M = 128,
// N = 2 NB, K = 16 per instruction).
//
// Throughput: on GB300 the tensor core's operand reads share the SM's
// shared memory with the S-tile stores and the panel copies: per 128 x 128
// tile and NB = 64, 64 KB of S written, 128 KB of operands read by the MMAs
// and a 32 KB panel, against 1,024 clocks of MMA issue at N = 128 and 512
// clocks of ex2 for the S values.  MMAs with N = 64 run at about half their
// peak rate on this part (67-95 clocks each against 32), so the panel is one
// N = 2 NB operand.  Measured (64 chunks x 64 RHS): tensor pipe 21% busy,
// shared-memory pipes 29% (LSU) and 23% (tensor core), issue 42%: the
// two-stage S pipeline leaves latency exposed rather than saturating a pipe.
//
// Precision: S and u = w p are split into BF16 hi + lo parts.  The u panel
// of a column tile is one B operand of N = 2 NB rows, [u_hi | u_lo], so two
// MMAs per K step (S_hi [u_hi | u_lo] and S_lo [u_hi | u_lo], N = 2 NB: wide
// MMAs run near the tensor pipe's peak where N = NB ones do not) accumulate
// D = [S u_hi | S u_lo] and the epilogue adds the halves: about 16
// significant bits per term with an FP32 accumulator, an operator error near
// 1e-5 relative, which the FP64 reliable updates of the solver remove.
//
// Per CTA (one per SM, GEN_WARPS + 2 warps, persistent over (row tile, RHS
// block) items), warp-specialized with mbarrier hand-offs:
//   * warps 0 .. GEN_WARPS - 1 generate S for the current column tile (row
//     sub-tile warp % 4, 128 / (GEN_WARPS / 4) columns per warp; EXPANDED
//     exponent: 3 FFMA + ex2 per pair; DIRECT when the tiles are too wide for
//     it), split it into BF16 hi / lo and store both into shared memory in
//     the canonical K-major no-swizzle layout (8 x 16-byte core matrices); a
//     32 x 32 sub-tile outside the cutoff is zero.  After an item's last tile
//     they read D back (tcgen05.ld; warp w may read TMEM lanes
//     32 (w % 4) .. + 31, its own rows), form q = rowf D + ediag p and the
//     tile's p.q per RHS;
//   * warp GEN_WARPS stages the column coordinates of each column tile and
//     issues the cp.async.bulk copy of its u panel (pre-packed in HBM by
//     k_pack_panels in the same core-matrix layout);
//   * lane 0 of warp GEN_WARPS + 1 issues the MMAs (K steps whose column
//     sub-tile interacts with no row sub-tile are skipped) and commits them;
//   * S tiles, panels and coordinates are double-buffered and the
//     accumulator has two TMEM buffers, so generation of tile g + 1 overlaps
//     the MMAs of tile g and an item's epilogue overlaps the next item.
// Every mbarrier wait is bounded: on a time-out the kernel records an error
// code, waits (bounded) for its own MMAs and copies, frees its tensor memory
// and returns.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdint>

#include "ds_batch.h"
#include "ds_tc.cuh"

namespace ds {
namespace {

constexpr int GEN_WARPS = 8;                       // S generation + epilogue (8 or 16)
constexpr int GEN_CW = GEN_WARPS / 4;              // warps per row sub-tile
constexpr int GEN_CS = 4 / GEN_CW;                 // column sub-tiles per warp
constexpr int TC_THREADS = (GEN_WARPS + 2) * 32;   // + producer warp + MMA warp
// One CTA per SM: the warps are spread over the 4 SM sub-partitions, each
// with 16,384 registers, so the busiest one holds ceil(warps / 4) warps.
constexpr int TC_MAXNREG = (16384 / (32 * ((TC_THREADS / 32 + 3) / 4))) & ~7;
__device__ __forceinline__ float ex2_tc(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// hi = bf16(a), lo = bf16(a - hi) for a pair, packed as bf16x2.
__device__ __forceinline__ void split2(float a, float b, uint32_t& hi, uint32_t& lo) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  const __nv_bfloat162 l =
      __floats2bfloat162_rn(a - __low2float(h), b - __high2float(h));
  hi = *reinterpret_cast<const uint32_t*>(&h);
  lo = *reinterpret_cast<const uint32_t*>(&l);
}

// Elements of one S buffer (128 x 128 BF16) and one u panel (NB x 128).
constexpr int S_ELEMS = TILE * TILE;
// Core-matrix layout (K-major, no swizzle), in BF16 elements: element
// (row m, k) of a 128-row operand at ((k / 8) * 16 + m / 8) * 64 + (m % 8) * 8
// + k % 8, i.e. LBO (K-adjacent) 2048 bytes, SBO (M-adjacent) 128 bytes.  A u
// panel has 2 NB rows n (u_hi of RHS n for n < NB, u_lo of RHS n - NB above)
// and k = pixel, at ((k / 8) * (2 NB / 8) + n / 8) * 64 + (n % 8) * 8 + k % 8:
// LBO 2 NB / 8 * 128 bytes, SBO 128 bytes.
constexpr uint32_t S_LBO = 16 * 128;
constexpr uint32_t CORE_SBO = 128;

template <int NB>
struct TcSmem {
  __nv_bfloat16 s[2][2][S_ELEMS];     // [buffer][hi, lo] generated S tiles
  __nv_bfloat16 u[2][2 * NB * TILE];  // [buffer] u panel, hi then lo
  float4 sc[2][TILE];                 // [buffer] column coordinates of the tile
  float red[2][GEN_WARPS][32];        // [D buffer][warp] per-column p.q sums
  uint64_t sc_full[2];   // column coordinates staged       (1 arrive)
  uint64_t u_full[2];    // u panel landed                  (1 arrive + tx bytes)
  uint64_t s_full[2];    // S tile written                  (GEN_WARPS arrives)
  uint64_t mma_done[2];  // MMAs reading buffer b completed (tcgen05.commit)
  uint64_t d_full[2];    // all MMAs of an item completed   (tcgen05.commit)
  uint64_t d_empty[2];   // D read back by the epilogue     (GEN_WARPS arrives)
  uint64_t red_full[2];  // per-warp column sums written    (GEN_WARPS arrives)
  uint32_t tmem_addr;
  int abort;
};

template <int NB>
constexpr size_t tc_smem_bytes() {
  return sizeof(TcSmem<NB>) + 1024;  // + alignment slack
}

// A bounded wait that records a time-out: error code, CTA abort flag.
template <int NB>
__device__ __forceinline__ bool wait_or_abort(TcSmem<NB>& sm, uint64_t* bar, uint32_t parity,
                                              int* err, int code, long long limit) {
  if (mbar_wait(bar, parity, limit)) return true;
  atomicExch(err, code);
  *(volatile int*)&sm.abort = 1;
  return false;
}

// The same for a whole warp: lane 0 polls (one shared-memory access per poll
// instead of 32) and the warp's barrier orders the other lanes' reads after
// the observed phase.
template <int NB>
__device__ __forceinline__ bool warp_wait_or_abort(TcSmem<NB>& sm, uint64_t* bar,
                                                   uint32_t parity, int* err, int code,
                                                   long long limit, int lane) {
  int ok = 1;
  if (lane == 0) ok = wait_or_abort(sm, bar, parity, err, code, limit);
  ok = __shfl_sync(0xffffffffu, ok, 0);
  __syncwarp();
  return ok != 0;
}

__device__ __forceinline__ bool aborted(const int* flag) { return *(const volatile int*)flag != 0; }

// Column sums over the warp's 32 rows of v[0..HN): afterwards lane l < HN
// holds the sum of column l (recursive halving: 31 shuffles for HN = 32).
template <int HN>
__device__ __forceinline__ float warp_column_sums(float (&v)[HN], int lane) {
#pragma unroll
  for (int s = HN / 2; s >= 1; s >>= 1) {
    const bool upper = (lane & s) != 0;
#pragma unroll
    for (int j = 0; j < s; ++j) {
      const float send = upper ? v[j] : v[j + s];
      const float keep = upper ? v[j + s] : v[j];
      v[j] = keep + __shfl_xor_sync(0xffffffffu, send, s);
    }
  }
  float r = v[0];
#pragma unroll
  for (int s = HN; s < 32; s <<= 1) r += __shfl_xor_sync(0xffffffffu, r, s);
  return r;
}

// Warp roles: warps 0 .. GEN_WARPS - 1 generate S and run the epilogue; warp
// GEN_WARPS stages the column coordinates and issues the u-panel copy of each
// column tile; lane 0 of warp GEN_WARPS + 1 issues the MMAs.  The
// hand-offs are mbarriers, so no role waits for another except for data:
// generation of tile g + 1 overlaps the MMAs of tile g, and the epilogue of
// an item (its accumulator in one of two TMEM buffers) overlaps the MMAs of
// the next.  Items are dealt round-robin (item = CTA + k * grid), in the
// launch order (chunks by decreasing work), so every role walks the same
// sequence without a queue.
template <int NB, int FORMULA>
__global__ void __maxnreg__(TC_MAXNREG) k_batch_mv_tc(BatchF32Args a) {
  static_assert(NB == 16 || NB == 32 || NB == 64, "RHS block");
  constexpr uint32_t D_COLS = 2 * NB;  // [S u_hi | S u_lo] per accumulator buffer
  constexpr uint32_t TMEM_COLS = 2 * D_COLS < 32 ? 32 : 2 * D_COLS;
  constexpr uint32_t PANEL_BYTES = 2u * NB * TILE * 2u;
  constexpr uint32_t U_LBO = (2 * NB / 8) * 128;
  constexpr uint32_t IDESC = idesc_bf16(128, 2 * NB);
  constexpr int HN = NB / GEN_CW;  // RHS columns of D per generation warp
  extern __shared__ uint8_t smem_raw[];
  TcSmem<NB>& sm = *reinterpret_cast<TcSmem<NB>*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int b = 0; b < 2; ++b) {
      mbar_init(&sm.sc_full[b], 1);
      mbar_init(&sm.u_full[b], 1);
      mbar_init(&sm.s_full[b], GEN_WARPS);
      mbar_init(&sm.mma_done[b], 1);
      mbar_init(&sm.d_full[b], 1);
      mbar_init(&sm.d_empty[b], GEN_WARPS);
      mbar_init(&sm.red_full[b], GEN_WARPS);
    }
    sm.abort = 0;
    mbar_fence_init();
  }
  if (warp == 0) tmem_alloc(&sm.tmem_addr, TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = sm.tmem_addr;
  const int R = a.n_rhs;
  const int nblk = R / NB;
  const int n_items = a.n_row_tiles * nblk;
  const __nv_bfloat16* panels = reinterpret_cast<const __nv_bfloat16*>(a.panel);
  int last_g = -1;  // last tile of this role's walk (MMA commit / panel copy in flight)

  if (warp < GEN_WARPS) {
    // ---- generation and epilogue ------------------------------------------
    // warp = 4 cw + rs: row sub-tile rs (TMEM lanes 32 rs ..), column
    // sub-tiles GEN_CS cw .. GEN_CS cw + GEN_CS - 1 of S, D columns cw HN ..
    // In generation lane l forms rows 32 rs + 8 j + (l & 7), j = 0..3, times
    // the 8 columns 8 (l >> 3) .. of each column sub-tile, so each staged
    // column is read once per 4 rows.  128-bit shared accesses are served
    // 8 lanes at a time: lanes 8q .. 8q + 7 read the same coordinates
    // (broadcast) and store 8 consecutive rows (128 contiguous bytes).  In
    // the epilogue lane l owns row 32 rs + l (its TMEM lane).
    const int rs = warp & 3, cw = warp >> 2;
    const int kq = lane >> 3, rl = lane & 7;
    const int row = 32 * rs + lane;
    uint32_t g = 0, k = 0;
    for (int item = blockIdx.x; item < n_items; item += gridDim.x) {
      const int t = a.row_order[item / nblk];
      const int rb = item % nblk;
      if (a.chunk_done[a.tile_chunk[t]]) continue;
      const int i = t * TILE + row;
      float4 me[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) me[j] = a.xi[t * TILE + 32 * rs + 8 * j + rl];
      const int p0 = a.row_ptr[t], p1 = a.row_ptr[t + 1];
      bool any = false;
      unsigned m = a.mask[p0];
      for (int p = p0; p < p1; ++p, ++g) {
        const uint32_t b = g & 1;
        const unsigned mnext = p + 1 < p1 ? a.mask[p + 1] : 0u;
        any |= m != 0u;
        // S values of this warp's sub-tiles are formed in registers as soon as
        // the coordinates are staged; the S buffer is awaited only for the
        // stores
        if (!warp_wait_or_abort(sm, &sm.sc_full[b], (g >> 1) & 1u, a.err, 11, a.wait_limit,
                                lane))
          break;
        const float4* sc = sm.sc[b];
        uint4 vh[GEN_CS][4], vl[GEN_CS][4];
#pragma unroll
        for (int c2 = 0; c2 < GEN_CS; ++c2) {
          const int cs = GEN_CS * cw + c2;
          const bool on = (m >> (4 * rs + cs)) & 1u;
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            vh[c2][j] = make_uint4(0u, 0u, 0u, 0u);
            vl[c2][j] = make_uint4(0u, 0u, 0u, 0u);
          }
          if (on) {
            const int kg = cs * 4 + kq;
            float sv[4][8];
#pragma unroll
            for (int e = 0; e < 8; ++e) {
              const float4 c4 = sc[kg * 8 + e];
#pragma unroll
              for (int j = 0; j < 4; ++j) {
                float t2;
                if (FORMULA == F32_EXPANDED) {
                  t2 = fmaf(me[j].x, c4.x, c4.w);
                  t2 = fmaf(me[j].y, c4.y, t2);
                  t2 = fmaf(me[j].z, c4.z, t2);
                } else {
                  const float dx = me[j].x - c4.x, dy = me[j].y - c4.y, dz = me[j].z - c4.z;
                  t2 = -fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                }
                sv[j][e] = ex2_tc(t2);
              }
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              split2(sv[j][0], sv[j][1], vh[c2][j].x, vl[c2][j].x);
              split2(sv[j][2], sv[j][3], vh[c2][j].y, vl[c2][j].y);
              split2(sv[j][4], sv[j][5], vh[c2][j].z, vl[c2][j].z);
              split2(sv[j][6], sv[j][7], vh[c2][j].w, vl[c2][j].w);
            }
          }
        }
        if (g >= 2 &&
            !warp_wait_or_abort(sm, &sm.mma_done[b], ((g >> 1) - 1) & 1u, a.err, 12,
                                a.wait_limit, lane))
          break;
        __nv_bfloat16* shi = sm.s[b][0];
        __nv_bfloat16* slo = sm.s[b][1];
#pragma unroll
        for (int c2 = 0; c2 < GEN_CS; ++c2) {
          const int kg = (GEN_CS * cw + c2) * 4 + kq;
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            // row 32 rs + 8 j + rl: 8-row group 4 rs + j, row rl within it
            const int off = (kg * 16 + 4 * rs + j) * 64 + rl * 8;
            *reinterpret_cast<uint4*>(shi + off) = vh[c2][j];
            *reinterpret_cast<uint4*>(slo + off) = vl[c2][j];
          }
        }
        fence_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(&sm.s_full[b]);
        m = mnext;
      }
      if (aborted(&sm.abort)) break;
      // epilogue: D of this item in TMEM buffer db; the row's p values and
      // coefficients are loaded before the wait
      const uint32_t db = k & 1;
      const float rf = a.rowf[i], ed = a.ediag[i];
      const int r0 = rb * NB + cw * HN;
      const float4* pv4 = reinterpret_cast<const float4*>(a.p + (size_t)i * R + r0);
      float4* qv4 = reinterpret_cast<float4*>(a.q + (size_t)i * R + r0);
      float4 pvr[HN / 4];
#pragma unroll
      for (int k4 = 0; k4 < HN / 4; ++k4) pvr[k4] = pv4[k4];
      if (!warp_wait_or_abort(sm, &sm.d_full[db], (k >> 1) & 1u, a.err, 13, a.wait_limit,
                              lane))
        break;
      __syncwarp();
      tc_fence_after();
      float d[HN], dl[HN];
      const uint32_t tl = tmem + ((uint32_t)(32 * rs) << 16) + db * D_COLS + (uint32_t)(cw * HN);
      tmem_ld<HN>(tl, d);        // S u_hi
      tmem_ld<HN>(tl + NB, dl);  // S u_lo
#pragma unroll
      for (int j = 0; j < HN; ++j) d[j] += dl[j];
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.d_empty[db]);
      if (!any) {
#pragma unroll
        for (int j = 0; j < HN; ++j) d[j] = 0.f;
      }
#pragma unroll
      for (int k4 = 0; k4 < HN / 4; ++k4) {
        const float4 pv = pvr[k4];
        float4 qv;
        qv.x = fmaf(rf, d[4 * k4 + 0], ed * pv.x);
        qv.y = fmaf(rf, d[4 * k4 + 1], ed * pv.y);
        qv.z = fmaf(rf, d[4 * k4 + 2], ed * pv.z);
        qv.w = fmaf(rf, d[4 * k4 + 3], ed * pv.w);
        qv4[k4] = qv;
        d[4 * k4 + 0] = pv.x * qv.x;  // d now holds the p.q products
        d[4 * k4 + 1] = pv.y * qv.y;
        d[4 * k4 + 2] = pv.z * qv.z;
        d[4 * k4 + 3] = pv.w * qv.w;
      }
      const float csum = warp_column_sums<HN>(d, lane);
      if (lane < HN) sm.red[db][warp][lane] = csum;
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.red_full[db]);
      // The sums of buffer db are read before this item's column sums of
      // buffer db are rewritten two items later: those need D of that item,
      // i.e. the S tiles of the item in between from every generation warp.
      if (warp < NB / 32 + (NB < 32) &&
          !warp_wait_or_abort(sm, &sm.red_full[db], (k >> 1) & 1u, a.err, 14, a.wait_limit,
                              lane))
        break;
      if (tid < NB) {
        // column tid of the block: warp column group h = tid / HN, summed
        // over the four row sub-tiles (warps 4 h .. 4 h + 3)
        const int h = tid / HN, j = tid % HN;
        double sum = 0.0;
#pragma unroll
        for (int w = 0; w < 4; ++w) sum += (double)sm.red[db][h * 4 + w][j];
        a.part[(size_t)t * R + rb * NB + tid] = sum;
      }
      if (a.prof_pairs && tid == 0) {
        unsigned long long n_sub = 0;
        for (int p = p0; p < p1; ++p) n_sub += __popc(a.mask[p]);
        atomicAdd(a.prof_pairs, n_sub * SUBTILE * SUBTILE * NB);
      }
      ++k;
    }
  } else if (warp == GEN_WARPS) {
    // ---- producer: column coordinates and u panels ------------------------------
    // The next tile's indices and coordinates are loaded into registers
    // before waiting for its buffer, so their latency overlaps that wait.
    uint32_t g = 0;
    for (int item = blockIdx.x; item < n_items; item += gridDim.x) {
      const int t = a.row_order[item / nblk];
      const int rb = item % nblk;
      if (a.chunk_done[a.tile_chunk[t]]) continue;
      const float4 ot = a.orig[t];
      const int p0 = a.row_ptr[t], p1 = a.row_ptr[t + 1];
      int ct = p0 < p1 ? a.cols[p0] : 0;
      float4 co = a.orig[ct];
      float4 cq[TILE / 32];
#pragma unroll
      for (int q = 0; q < TILE / 32; ++q) cq[q] = a.xi[ct * TILE + lane + 32 * q];
      for (int p = p0; p < p1; ++p, ++g) {
        const uint32_t b = g & 1;
        if (aborted(&sm.abort)) break;
        // prefetch of tile p + 1
        const int ct_n = p + 1 < p1 ? a.cols[p + 1] : ct;
        const float4 co_n = a.orig[ct_n];
        float4 cq_n[TILE / 32];
#pragma unroll
        for (int q = 0; q < TILE / 32; ++q) cq_n[q] = a.xi[ct_n * TILE + lane + 32 * q];
        // sc[b] is free once every generation warp finished tile g - 2
        if (g >= 2 &&
            !warp_wait_or_abort(sm, &sm.s_full[b], ((g >> 1) - 1) & 1u, a.err, 22,
                                a.wait_limit, lane))
          break;
#pragma unroll
        for (int q = 0; q < TILE / 32; ++q) {
          const int col = lane + 32 * q;
          const float zx = cq[q].x - (ot.x - co.x), zy = cq[q].y - (ot.y - co.y);
          const float zz = cq[q].z - (ot.z - co.z);
          if (FORMULA == F32_EXPANDED)
            sm.sc[b][col] =
                make_float4(2.f * zx, 2.f * zy, 2.f * zz, -fmaf(zx, zx, fmaf(zy, zy, zz * zz)));
          else
            sm.sc[b][col] = make_float4(zx, zy, zz, 0.f);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&sm.sc_full[b]);
        // u[b] is free once the MMAs of tile g - 2 completed
        if (g >= 2 &&
            !warp_wait_or_abort(sm, &sm.mma_done[b], ((g >> 1) - 1) & 1u, a.err, 21,
                                a.wait_limit, lane))
          break;
        if (lane == 0) {
          mbar_expect_tx(&sm.u_full[b], PANEL_BYTES);
          bulk_g2s(sm.u[b], panels + ((size_t)ct * nblk + rb) * (2 * NB * TILE), PANEL_BYTES,
                   &sm.u_full[b]);
        }
        last_g = (int)g;
        ct = ct_n;
        co = co_n;
#pragma unroll
        for (int q = 0; q < TILE / 32; ++q) cq[q] = cq_n[q];
      }
      if (aborted(&sm.abort)) break;
    }
  } else if (lane == 0) {
    // ---- MMA issue ------------------------------------------------------------
    uint32_t g = 0, k = 0;
    for (int item = blockIdx.x; item < n_items; item += gridDim.x) {
      const int t = a.row_order[item / nblk];
      if (a.chunk_done[a.tile_chunk[t]]) continue;
      const int p0 = a.row_ptr[t], p1 = a.row_ptr[t + 1];
      const uint32_t db = k & 1;
      if (k >= 2 && !wait_or_abort(sm, &sm.d_empty[db], ((k >> 1) - 1) & 1u, a.err, 31,
                                   a.wait_limit))
        break;
      tc_fence_after();
      const uint32_t dt = tmem + db * D_COLS;
      uint32_t accumulate = 0;
      bool ok = true;
      for (int p = p0; p < p1; ++p, ++g) {
        const uint32_t b = g & 1;
        if (!wait_or_abort(sm, &sm.u_full[b], (g >> 1) & 1u, a.err, 32, a.wait_limit) ||
            !wait_or_abort(sm, &sm.s_full[b], (g >> 1) & 1u, a.err, 33, a.wait_limit)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const unsigned m = a.mask[p];
        const uint32_t sa = smem_u32(sm.s[b][0]), sl = smem_u32(sm.s[b][1]);
        const uint32_t ua = smem_u32(sm.u[b]);
#pragma unroll 1
        for (int ks = 0; ks < TILE / 16; ++ks) {
          if (!((m >> (ks >> 1)) & 0x1111u)) continue;  // no row sub-tile reaches it
          const uint32_t aoff = ks * 2 * S_LBO, boff = ks * 2 * U_LBO;
          const uint64_t ahi = sdesc(sa + aoff, S_LBO, CORE_SBO);
          const uint64_t alo = sdesc(sl + aoff, S_LBO, CORE_SBO);
          const uint64_t bu = sdesc(ua + boff, U_LBO, CORE_SBO);
          mma_bf16(dt, ahi, bu, IDESC, accumulate);
          mma_bf16(dt, alo, bu, IDESC, 1u);
          accumulate = 1u;
        }
        mma_commit(&sm.mma_done[b]);
        last_g = (int)g;
      }
      if (!ok) break;
      mma_commit(&sm.d_full[db]);
      ++k;
    }
  }
  // teardown: after a time-out, wait (bounded by the default, whatever the
  // caller's limit) for this role's work in flight before the tensor memory
  // and the shared memory are released: the last MMA commit (it covers every
  // earlier MMA of the thread) and the last two panel copies (a copy into a
  // buffer is issued only after the copy before it in that buffer was used).
  if (aborted(&sm.abort) && last_g >= 0 && lane == 0) {
    if (warp == GEN_WARPS) {
      mbar_wait(&sm.u_full[last_g & 1], (last_g >> 1) & 1u);
      if (last_g >= 1) mbar_wait(&sm.u_full[(last_g - 1) & 1], ((last_g - 1) >> 1) & 1u);
    }
    if (warp == GEN_WARPS + 1) mbar_wait(&sm.mma_done[last_g & 1], (last_g >> 1) & 1u);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, TMEM_COLS);
}

// u = colw p as BF16 hi / lo panels: per (column tile, RHS block of NB), one
// 2 NB-row operand [u_hi | u_lo] in the core-matrix layout above.  One
// thread per (tile, group of 8 pixels, RHS): 8 strided reads (coalesced over
// the RHS index), one 16-byte store per part.
template <int NB>
__global__ void k_pack_panels(int n_tiles, int R, const float* __restrict__ p,
                              const float* __restrict__ colw, __nv_bfloat16* __restrict__ panel) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t total = (size_t)n_tiles * (TILE / 8) * R;
  if (k >= total) return;
  const int r = (int)(k % R);
  const size_t tk = k / R;
  const int kg = (int)(tk % (TILE / 8));
  const int ct = (int)(tk / (TILE / 8));
  const int j0 = ct * TILE + kg * 8;
  float u[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) u[e] = colw[j0 + e] * p[(size_t)(j0 + e) * R + r];
  uint4 vh, vl;
  split2(u[0], u[1], vh.x, vl.x);
  split2(u[2], u[3], vh.y, vl.y);
  split2(u[4], u[5], vh.z, vl.z);
  split2(u[6], u[7], vh.w, vl.w);
  const int rb = r / NB, rr = r % NB;
  const size_t base = ((size_t)ct * (R / NB) + rb) * (2 * NB * TILE);
  const int offh = (kg * (2 * NB / 8) + rr / 8) * 64 + (rr % 8) * 8;
  const int offl = (kg * (2 * NB / 8) + (NB + rr) / 8) * 64 + (rr % 8) * 8;
  *reinterpret_cast<uint4*>(panel + base + offh) = vh;
  *reinterpret_cast<uint4*>(panel + base + offl) = vl;
}

template <int NB, int FORMULA>
void tc_launch(const BatchF32Args& a, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    DS_CUDA(cudaFuncSetAttribute(k_batch_mv_tc<NB, FORMULA>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)tc_smem_bytes<NB>()));
    attr = true;
  }
  const size_t packs = (size_t)a.n_row_tiles * (TILE / 8) * a.n_rhs;
  k_pack_panels<NB><<<(unsigned)((packs + 255) / 256), 256, 0, st>>>(
      a.n_row_tiles, a.n_rhs, a.p, a.colw, reinterpret_cast<__nv_bfloat16*>(a.panel));
  DS_CHECK_LAUNCH();
  static int sms = 0;  // queried on the first (uncaptured) launch
  if (!sms) {
    int dev = 0;
    DS_CUDA(cudaGetDevice(&dev));
    DS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  }
  const int items = a.n_row_tiles * (a.n_rhs / NB);
  const int grid = std::max(1, std::min(items, sms));
  k_batch_mv_tc<NB, FORMULA><<<grid, TC_THREADS, tc_smem_bytes<NB>(), st>>>(a);
  DS_CHECK_LAUNCH();
}

}  // namespace

int batch_tc_block(int R) {
  if (R % 64 == 0) return 64;
  if (R % 32 == 0) return 32;
  if (R % 16 == 0) return 16;
  return 0;
}

size_t batch_tc_panel_elems(int n_tiles, int R) { return (size_t)n_tiles * TILE * R * 2; }

template <int FORMULA>
void tc_dispatch(const BatchF32Args& a, cudaStream_t st) {
  switch (batch_tc_block(a.n_rhs)) {
    case 64: tc_launch<64, FORMULA>(a, st); break;
    case 32: tc_launch<32, FORMULA>(a, st); break;
    case 16: tc_launch<16, FORMULA>(a, st); break;
    default: throw Error{DS_ERR_ARG, "the tensor-core matvec needs n_rhs % 16 == 0"};
  }
}

void launch_batch_mv_tc(const BatchF32Args& a, cudaStream_t st) {
  if (a.formula == F32_EXPANDED)
    tc_dispatch<F32_EXPANDED>(a, st);
  else
    tc_dispatch<F32_DIRECT>(a, st);
}

}  // namespace ds
