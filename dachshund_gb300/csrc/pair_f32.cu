// FP32 matrix-free pair kernels of the mixed-precision form: the exact
// kernel var_s exp(-arg) evaluated as var_s 2^(-|dX|^2) on coordinates scaled
// by sqrt(c log2 e), with MUFU ex2 and packed f32x2 FMAs.
//
// Coordinates are stored relative to their tile's origin (the bounding-box
// centre, rounded to FP32), so FP32 differences are taken between numbers of
// the size of a tile rather than of the box.  For a (row tile R, column tile
// C) pair the columns are moved into R's frame once at staging:
//   zeta_j = xi_j - (o_R - o_C).
// Two formulations of the exponent:
//   EXPANDED  t_ij = 2 xi_i . zeta_j - |zeta_j|^2 = |xi_i|^2 - |xi_i - zeta_j|^2,
//             e_ij = 2^t_ij = 2^(|xi_i|^2) S'_ij, the row factor 2^-|xi_i|^2
//             applied once at the end.  Per pair: 3 FFMA + 1 ex2 + 1 FFMA,
//             i.e. 4 FMA-pipe lanes and 1 MUFU: FMA and MUFU (both 32/clk/SM
//             on GB300) are co-bound at 32 pairs/clk/SM.  Relative error of
//             S' about |zeta|^2 * 2^-24 (~1e-6): used for the inner solve,
//             whose FP64 outer residual removes it.
//   DIRECT    t_ij = -|xi_i - zeta_j|^2: 3 FADD + FMUL + 2 FFMA + ex2 + FFMA,
//             7 FMA-pipe lanes (18 pairs/clk/SM); relative error ~1e-7.  Used
//             for the map product and when a tile is too large for EXPANDED
//             (2^|xi|^2 would leave FP32 range).
// Each CTA owns a 128-row tile; lane l of each warp holds rows l, l+32, l+64,
// l+96 (as two f32x2 pairs), and the warps share out the row tile's work
// items (32-column sub-tiles of its interacting column tiles), staging two
// items per round, so a staged column is read once per 4 rows.  Each round's
// FP32 sums (64 terms; 32 for the map, which folds each item on its own) are
// folded into Kahan-compensated FP32 accumulators; the four warps' partial
// rows are summed in FP64 at the end.
#include "ds_device.cuh"
#include "ds_f32.h"

namespace ds {

namespace {

// CTAs per SM the register budget is sized for (4 warps each): 96 registers
// hold the two prefetched column tiles and a fully unrolled 32-column loop;
// on the 262,144-pixel workload 5 CTAs per SM beat 4, 6, 7 (with spills) and
// the one-tile prefetch at 8.
constexpr int F32_MIN_CTAS = 5;

__device__ __forceinline__ float ex2f(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ void kahan_add(float& s, float& c, float v) {
  const float y = v - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

// One warp's 32 staged columns against its lane's four rows, as two f32x2 row
// pairs (01: rows lane and lane+32, 23: rows lane+64 and lane+96).  A pair
// whose two row sub-tiles are both beyond the cutoff from the column
// sub-tile is skipped (DO01 / DO23 false).  The column values come four to a
// shared-memory load.
template <int FORMULA, bool DO01, bool DO23>
__device__ __forceinline__ void accumulate32(const float4* __restrict__ col,
                                             const float4* __restrict__ cu4, float2 x01,
                                             float2 y01, float2 z01, float2 x23, float2 y23,
                                             float2 z23, float2& acc01, float2& acc23) {
#pragma unroll
  for (int qd = 0; qd < 8; ++qd) {
    const float4 u4 = cu4[qd];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float4 c4 = col[4 * qd + k];
      const float uk = k == 0 ? u4.x : k == 1 ? u4.y : k == 2 ? u4.z : u4.w;
      const float2 u2 = make_float2(uk, uk);
      float2 t01, t23;
      if (FORMULA == F32_EXPANDED) {
        const float2 cx = make_float2(c4.x, c4.x), cy = make_float2(c4.y, c4.y);
        const float2 cz = make_float2(c4.z, c4.z), cw = make_float2(c4.w, c4.w);
        if (DO01) {
          t01 = __ffma2_rn(x01, cx, cw);
          t01 = __ffma2_rn(y01, cy, t01);
          t01 = __ffma2_rn(z01, cz, t01);
        }
        if (DO23) {
          t23 = __ffma2_rn(x23, cx, cw);
          t23 = __ffma2_rn(y23, cy, t23);
          t23 = __ffma2_rn(z23, cz, t23);
        }
      } else {
        const float2 ncx = make_float2(-c4.x, -c4.x), ncy = make_float2(-c4.y, -c4.y);
        const float2 ncz = make_float2(-c4.z, -c4.z);
        if (DO01) {
          const float2 dx = __fadd2_rn(x01, ncx), dy = __fadd2_rn(y01, ncy);
          const float2 dz = __fadd2_rn(z01, ncz);
          t01 = __fmul2_rn(dx, make_float2(-dx.x, -dx.y));
          t01 = __ffma2_rn(dy, make_float2(-dy.x, -dy.y), t01);
          t01 = __ffma2_rn(dz, make_float2(-dz.x, -dz.y), t01);
        }
        if (DO23) {
          const float2 dx = __fadd2_rn(x23, ncx), dy = __fadd2_rn(y23, ncy);
          const float2 dz = __fadd2_rn(z23, ncz);
          t23 = __fmul2_rn(dx, make_float2(-dx.x, -dx.y));
          t23 = __ffma2_rn(dy, make_float2(-dy.x, -dy.y), t23);
          t23 = __ffma2_rn(dz, make_float2(-dz.x, -dz.y), t23);
        }
      }
      if (DO01) acc01 = __ffma2_rn(make_float2(ex2f(t01.x), ex2f(t01.y)), u2, acc01);
      if (DO23) acc23 = __ffma2_rn(make_float2(ex2f(t23.x), ex2f(t23.y)), u2, acc23);
    }
  }
}

// The 32 columns of one staged work item with the row pairs its mask names.
template <int FORMULA>
__device__ __forceinline__ void accumulate_item(unsigned m, const float4* __restrict__ col,
                                                const float4* __restrict__ cu4, float2 x01,
                                                float2 y01, float2 z01, float2 x23, float2 y23,
                                                float2 z23, float2& acc01, float2& acc23) {
  const bool do01 = (m & 3u) != 0;   // row sub-tile 0 or 1
  const bool do23 = (m & 12u) != 0;  // row sub-tile 2 or 3
  if (do01 && do23)
    accumulate32<FORMULA, true, true>(col, cu4, x01, y01, z01, x23, y23, z23, acc01, acc23);
  else if (do01)
    accumulate32<FORMULA, true, false>(col, cu4, x01, y01, z01, x23, y23, z23, acc01, acc23);
  else if (do23)
    accumulate32<FORMULA, false, true>(col, cu4, x01, y01, z01, x23, y23, z23, acc01, acc23);
}

template <int FORMULA, int EPI, bool DOT>
__global__ void __launch_bounds__(TILE, F32_MIN_CTAS) k_pair_f32(F32Args a) {
  if (a.skip_flag && *a.skip_flag) return;
  // per warp: two staged work items (64 columns) and their column values
  __shared__ float4 sc[2 * TILE];
  __shared__ float4 su4[2 * TILE / 4];
  __shared__ float sred[4][TILE];
  __shared__ double red[TILE / 32];
  const int t = a.row_order ? a.row_order[blockIdx.x] : blockIdx.x;  // heaviest tiles first
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int base = t * TILE;

  float2 x01, y01, z01, x23, y23, z23;
  {
    const float4 r0 = a.rxi[base + lane], r1 = a.rxi[base + lane + 32];
    const float4 r2 = a.rxi[base + lane + 64], r3 = a.rxi[base + lane + 96];
    x01 = make_float2(r0.x, r1.x); y01 = make_float2(r0.y, r1.y); z01 = make_float2(r0.z, r1.z);
    x23 = make_float2(r2.x, r3.x); y23 = make_float2(r2.y, r3.y); z23 = make_float2(r2.z, r3.z);
  }
  const float4 ot = a.rorig[t];
  float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
  float c0 = 0.f, c1 = 0.f, c2 = 0.f, c3 = 0.f;
  unsigned evaluated = 0;  // pairs this warp evaluates (profiling; < 2^32 per warp)

  // Work items (column tile, column sub-tile w) of this row tile, in the
  // order of the tile pairs and then w (build_slice_items); warp v takes
  // items v, v + 4, v + 8, ...: the four warps carry equal work whatever the
  // masks (each warp sums all 128 rows, so the sub-tiles may be shared out
  // freely) and the order of every FP32 sum is fixed.  A warp reads its next
  // 32 items in one load (lane l: its item 32 b + l, the next batch
  // prefetched).  A round stages two items (64 columns, one per lane and
  // item) and folds them into the compensated sums once; the column inputs
  // of the next round are loaded into registers while a round is computed.
  const int i1 = a.item_ptr[t + 1];
  struct ColRegs {
    float3 q, o;   // this lane's column (tile-relative) and the tile's origin
    float u;       // colw v (product) or v (map)
    unsigned m;    // row sub-tiles interacting with the item's columns (bit k)
  };
  auto load = [&](ColRegs& c, unsigned it) {
    const int ct = (int)(it >> 6);
    const int j = ct * TILE + 32 * (int)((it >> 4) & 3u) + lane;
    const float4 o = a.corig[ct], q = a.cxi[j];
    c.o = make_float3(o.x, o.y, o.z);
    c.q = make_float3(q.x, q.y, q.z);
    c.u = (EPI == EPI_PRODUCT) ? a.colw[j] * a.v[j] : a.v[j];
    c.m = it & 15u;
  };
  constexpr unsigned full = 0xffffffffu;
  int nb = a.item_ptr[t] + warp;  // this warp's first item of the next batch
  unsigned nitem = nb + 4 * lane < i1 ? a.items[nb + 4 * lane] : 0u;
  unsigned witem = 0;  // this lane's item of the current batch
  int pos = 0, cnt = 0;  // items taken / held of the current batch
  auto fetch = [&](ColRegs& c) -> bool {
    if (pos == cnt) {
      if (nb >= i1) return false;
      cnt = min(32, (i1 - nb + 3) >> 2);
      pos = 0;
      witem = nitem;
      nb += 128;
      nitem = nb + 4 * lane < i1 ? a.items[nb + 4 * lane] : 0u;
    }
    load(c, __shfl_sync(full, witem, pos));
    ++pos;
    return true;
  };
  // Each warp stages and reads only its own 64 columns, so the warps of a
  // CTA never wait for each other inside the loop.
  float4* const scw = sc + warp * 64;
  float* const suw = reinterpret_cast<float*>(su4 + warp * 16);
  auto stage = [&](const ColRegs& c, int slot) {
    const float dx = ot.x - c.o.x, dy = ot.y - c.o.y, dz = ot.z - c.o.z;
    const float zx = c.q.x - dx, zy = c.q.y - dy, zz = c.q.z - dz;
    if (FORMULA == F32_EXPANDED) {
      const float aj = fmaf(zx, zx, fmaf(zy, zy, zz * zz));
      scw[slot + lane] = make_float4(2.f * zx, 2.f * zy, 2.f * zz, -aj);
    } else {
      scw[slot + lane] = make_float4(zx, zy, zz, 0.f);
    }
    suw[slot + lane] = c.u;
  };
  ColRegs ca, cb;
  bool va = fetch(ca);
  bool vb = va && fetch(cb);
  while (va) {
    const unsigned ma = ca.m, mb = vb ? cb.m : 0u;
    __syncwarp();
    stage(ca, 0);
    if (vb) stage(cb, 32);
    __syncwarp();
    const bool na = vb && fetch(ca);
    const bool nbv = na && fetch(cb);
    if (a.prof_pairs)
      evaluated += 2 * SUBTILE * 32 * (((ma & 3u) != 0) + ((ma & 12u) != 0) +
                                       ((mb & 3u) != 0) + ((mb & 12u) != 0));
    float2 acc01 = make_float2(0.f, 0.f), acc23 = make_float2(0.f, 0.f);
    accumulate_item<FORMULA>(ma, scw, su4 + warp * 16, x01, y01, z01, x23, y23, z23, acc01,
                             acc23);
    if (EPI == EPI_MAP) {
      // the map keeps 32-term FP32 partials: each item is folded on its own
      kahan_add(s0, c0, acc01.x);
      kahan_add(s1, c1, acc01.y);
      kahan_add(s2, c2, acc23.x);
      kahan_add(s3, c3, acc23.y);
      acc01 = make_float2(0.f, 0.f);
      acc23 = make_float2(0.f, 0.f);
    }
    accumulate_item<FORMULA>(mb, scw + 32, su4 + warp * 16 + 8, x01, y01, z01, x23, y23, z23,
                             acc01, acc23);
    kahan_add(s0, c0, acc01.x);
    kahan_add(s1, c1, acc01.y);
    kahan_add(s2, c2, acc23.x);
    kahan_add(s3, c3, acc23.y);
    va = na;
    vb = nbv;
  }
  if (a.prof_pairs && lane == 0) atomicAdd(a.prof_pairs, (unsigned long long)evaluated);
  // Cross-warp reduction of the four column slices, in FP64.
  sred[warp][lane] = s0 - c0;
  sred[warp][lane + 32] = s1 - c1;
  sred[warp][lane + 64] = s2 - c2;
  sred[warp][lane + 96] = s3 - c3;
  __syncthreads();
  const double sum = ((double)sred[0][tid] + (double)sred[1][tid]) +
                     ((double)sred[2][tid] + (double)sred[3][tid]);
  const int i = base + tid;
  if (EPI == EPI_PRODUCT) {
    // q_i = wl_i var_s 2^-a_i sum_j e_ij wr_j v_j + e_i v_i
    const float q = fmaf(a.rowf[i], (float)sum, a.ediag[i] * a.vrow[i]);
    a.out[i] = q;
    if (DOT) {
      const double s = block_sum<TILE>((double)a.dotv[i] * (double)q, red);
      if (tid == 0) a.dot_partial[t] = s;
      if (last_block_arrive(a.counter)) {
        const double pq = reduce_partials<TILE>(a.dot_partial, gridDim.x, 1, 0, red);
        if (tid == 0) {
          *a.den_out = pq;
          *a.alpha_out = *a.num / pq;
          *a.counter = 0;
        }
      }
    }
  } else {
    // map: m_i = var_s * row factor * sum, accumulated in FP64
    const int dst = a.row_perm[i];
    if (dst >= 0) a.out64[dst] = (double)a.rowf[i] * sum;
  }
}

template <int FORMULA>
void launch_formula(int epi, const F32Args& a, cudaStream_t st) {
  const dim3 grid(a.n_row_tiles), block(TILE);
  if (epi == EPI_PRODUCT) {
    if (a.dot_partial)
      k_pair_f32<FORMULA, EPI_PRODUCT, true><<<grid, block, 0, st>>>(a);
    else
      k_pair_f32<FORMULA, EPI_PRODUCT, false><<<grid, block, 0, st>>>(a);
  } else if (epi == EPI_MAP) {
    k_pair_f32<FORMULA, EPI_MAP, false><<<grid, block, 0, st>>>(a);
  } else {
    throw Error{DS_ERR_ARG, "bad FP32 pair epilogue"};
  }
}

}  // namespace

void launch_pair_f32(int formula, int epi, const F32Args& a0, cudaStream_t st) {
  if (a0.n_row_tiles <= 0) return;
  F32Args a = a0;
  cudaEvent_t ev = nullptr;
  const int kind = epi == EPI_MAP ? 2 : 1;
  if (a.prof && a.prof->enabled) {
    a.prof_pairs = a.prof->d_pairs + kind;
    a.prof->begin(st, &ev);
  } else {
    a.prof_pairs = nullptr;
  }
  if (formula == F32_EXPANDED)
    launch_formula<F32_EXPANDED>(epi, a, st);
  else
    launch_formula<F32_DIRECT>(epi, a, st);
  DS_CHECK_LAUNCH();
  if (ev) a.prof->end(st, ev, kind);
}

}  // namespace ds
