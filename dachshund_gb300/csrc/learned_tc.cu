// Inference GEMMs of the learned preconditioner's message-passing layers on
// the tensor cores: out = res + relu(Z), Z = A W + b, with A the aggregated
// activations [M x 384] (FP32, row-major), W [384 x 128] (the BF16 forward
// weights, exact in TF32) and M a multiple of 128.  tcgen05.mma kind::tf32
// (M = N = 128, K = 8): the activations enter as TF32 (10-bit mantissa), a
// relative perturbation near 1e-3 of the hidden state against the FP32
// CUDA-core GEMM that training uses (whose gradients the CPU oracle checks);
// the preconditioner built from it differs correspondingly little, and the
// solve it preconditions still stops on its FP64-accurate residual.
//
// Per CTA (one per SM, persistent over 128-row tiles):
//   * warps 0-3 load K chunks of 32 (A rows of the tile and W^T rows) into 4
//     shared-memory stages in the canonical K-major no-swizzle layout; a
//     chunk's loads are in flight while the previous one is stored;
//   * lane 0 of warp 8 issues 4 MMAs per chunk into one of two TMEM
//     accumulators (128 columns each) and commits them;
//   * warps 4-7 read an accumulator back (warp w: TMEM lanes 32 (w % 4) ..,
//     its rows), add the bias, apply relu and the residual and store Z and
//     out, overlapping the next tile's MMAs.
// Every mbarrier wait is bounded (error code, then a clean exit).
#include "ds_device.cuh"
#include "ds_learned.h"
#include "ds_tc.cuh"

#include <cuda_bf16.h>

#include <algorithm>

namespace ds {
namespace {

constexpr int LG_K = 384;            // 3 H
constexpr int LG_N = 128;            // H
constexpr int LG_KC = 32;            // K per stage
constexpr int LG_NCH = LG_K / LG_KC;
constexpr int LG_STAGES = 4;
constexpr int LG_THREADS = 9 * 32;
constexpr int LG_OPF = 128 * LG_KC;  // floats of one 128-row operand chunk (16 KB)
constexpr uint32_t LG_LBO = 16 * 128;
constexpr uint32_t LG_SBO = 128;
constexpr uint32_t LG_IDESC = idesc_tf32(128, LG_N);

struct LgSmem {
  float a[LG_STAGES][LG_OPF];
  float b[LG_STAGES][LG_OPF];
  uint64_t full[LG_STAGES], empty[LG_STAGES];
  uint64_t d_full[2], d_empty[2];
  uint32_t tmem_addr;
  int abort;
};
constexpr size_t LG_SMEM_BYTES = sizeof(LgSmem) + 1024;

// element (row r, k) of a 128-row chunk with K = 32 (8 core-matrix columns)
__device__ __forceinline__ int lg_at(int r, int k) {
  return ((k >> 2) * 16 + (r >> 3)) * 32 + (r & 7) * 4 + (k & 3);
}

__device__ __forceinline__ bool lg_wait(LgSmem& sm, uint64_t* bar, uint32_t parity, int* err,
                                        int code) {
  if (mbar_wait(bar, parity)) return true;
  atomicExch(err, code);
  *(volatile int*)&sm.abort = 1;
  return false;
}

__device__ __forceinline__ bool lg_warp_wait(LgSmem& sm, uint64_t* bar, uint32_t parity,
                                             int* err, int code, int lane) {
  int ok = 1;
  if (lane == 0) ok = lg_wait(sm, bar, parity, err, code);
  ok = __shfl_sync(0xffffffffu, ok, 0);
  __syncwarp();
  return ok != 0;
}

// W^T as FP32 [128 x 384] row-major from the BF16 forward weights [384 x 128].
__global__ void k_wt_f32(const __nv_bfloat16* __restrict__ w, float* __restrict__ wt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= LG_K * LG_N) return;
  const int k = i / LG_N, n = i % LG_N;
  wt[(size_t)n * LG_K + k] = __bfloat162float(w[i]);
}

__global__ void __launch_bounds__(LG_THREADS, 1)
    k_layer_tc(int M, const float* __restrict__ A, const float* __restrict__ wt,
               const float* __restrict__ bias, float* __restrict__ Z, float* __restrict__ out,
               const float* __restrict__ res, int* err) {
  extern __shared__ uint8_t lg_raw[];
  LgSmem& sm = *reinterpret_cast<LgSmem*>((reinterpret_cast<uintptr_t>(lg_raw) + 1023) &
                                          ~uintptr_t(1023));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int s = 0; s < LG_STAGES; ++s) {
      mbar_init(&sm.full[s], 4);
      mbar_init(&sm.empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&sm.d_full[b], 1);
      mbar_init(&sm.d_empty[b], 4);
    }
    sm.abort = 0;
    mbar_fence_init();
  }
  if (warp == 0) tmem_alloc(&sm.tmem_addr, 256);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = sm.tmem_addr;
  const int n_tiles = M / 128;
  int last = -1;

  if (warp < 4) {
    // ---- producers: thread = row of the A chunk and row of the W^T chunk ----
    const int r = tid;
    uint32_t g = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
      const float4* arow = reinterpret_cast<const float4*>(A + ((size_t)tile * 128 + r) * LG_K);
      const float4* brow = reinterpret_cast<const float4*>(wt + (size_t)r * LG_K);
      float4 va[8], vb[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        va[q] = arow[q];
        vb[q] = brow[q];
      }
      for (int c = 0; c < LG_NCH; ++c, ++g) {
        const uint32_t s = g % LG_STAGES;
        if (g >= LG_STAGES &&
            !lg_warp_wait(sm, &sm.empty[s], ((g / LG_STAGES) - 1) & 1u, err, 71, lane)) {
          ok = false;
          break;
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          *reinterpret_cast<float4*>(&sm.a[s][lg_at(r, 4 * q)]) = va[q];
          *reinterpret_cast<float4*>(&sm.b[s][lg_at(r, 4 * q)]) = vb[q];
        }
        fence_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(&sm.full[s]);
        if (c + 1 < LG_NCH) {
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            va[q] = arow[8 * (c + 1) + q];
            vb[q] = brow[8 * (c + 1) + q];
          }
        }
      }
    }
  } else if (warp < 8) {
    // ---- epilogue -----------------------------------------------------------
    const int rs = warp & 3;
    uint32_t k = 0;
    for (int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x, ++k) {
      const uint32_t db = k & 1;
      if (!lg_warp_wait(sm, &sm.d_full[db], (k >> 1) & 1u, err, 72, lane)) break;
      tc_fence_after();
      const size_t m = (size_t)tile * 128 + 32 * rs + lane;
#pragma unroll 1
      for (int j = 0; j < LG_N / 32; ++j) {
        float d[32];
        tmem_ld<32>(tmem + ((uint32_t)(32 * rs) << 16) + db * 128u + 32u * j, d);
        const float4* b4 = reinterpret_cast<const float4*>(bias + 32 * j);
        const float4* r4 = reinterpret_cast<const float4*>(res + m * LG_N + 32 * j);
        float4* z4 = Z ? reinterpret_cast<float4*>(Z + m * LG_N + 32 * j) : nullptr;
        float4* o4 = reinterpret_cast<float4*>(out + m * LG_N + 32 * j);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const float4 bb = b4[q], rr = r4[q];
          const float4 zz = make_float4(d[4 * q] + bb.x, d[4 * q + 1] + bb.y, d[4 * q + 2] + bb.z,
                                        d[4 * q + 3] + bb.w);
          if (Z) z4[q] = zz;
          o4[q] = make_float4(rr.x + fmaxf(zz.x, 0.f), rr.y + fmaxf(zz.y, 0.f),
                              rr.z + fmaxf(zz.z, 0.f), rr.w + fmaxf(zz.w, 0.f));
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.d_empty[db]);
    }
  } else if (lane == 0) {
    // ---- MMA issue ------------------------------------------------------------
    uint32_t g = 0, k = 0;
    for (int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x, ++k) {
      const uint32_t db = k & 1;
      if (k >= 2 && !lg_wait(sm, &sm.d_empty[db], ((k >> 1) - 1) & 1u, err, 73)) break;
      tc_fence_after();
      bool ok = true;
      for (int c = 0; c < LG_NCH; ++c, ++g) {
        const uint32_t s = g % LG_STAGES;
        if (!lg_wait(sm, &sm.full[s], (g / LG_STAGES) & 1u, err, 74)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t sa = smem_u32(sm.a[s]), sb = smem_u32(sm.b[s]);
#pragma unroll
        for (int kk = 0; kk < LG_KC / 8; ++kk) {
          const uint64_t ad = sdesc(sa + kk * 2 * LG_LBO, LG_LBO, LG_SBO);
          const uint64_t bd = sdesc(sb + kk * 2 * LG_LBO, LG_LBO, LG_SBO);
          mma_tf32(tmem + db * 128u, ad, bd, LG_IDESC, (c > 0 || kk > 0) ? 1u : 0u);
        }
        mma_commit(&sm.empty[s]);
        last = (int)g;
      }
      if (!ok) break;
      mma_commit(&sm.d_full[db]);
    }
  }
  if (warp == 8 && lane == 0 && *(volatile int*)&sm.abort && last >= 0)
    mbar_wait(&sm.empty[last % LG_STAGES], (last / LG_STAGES) & 1u);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, 256);
}

}  // namespace

bool layer_tc_usable(int M, int N, int K) { return N == LG_N && K == LG_K && M % 128 == 0; }

// out = res + relu(Z), Z = A W + b for a message-passing layer (TF32 tensor
// cores); Z is stored only when given (training keeps it for the backward
// pass, inference does not); wt: scratch for W^T (LG_N x LG_K floats), err:
// device error flag.
void launch_layer_tc(int M, const float* A, const __nv_bfloat16* W, const float* bias, float* Z,
                     float* out, const float* res, float* wt, int* err, cudaStream_t st) {
  k_wt_f32<<<(LG_K * LG_N + 255) / 256, 256, 0, st>>>(W, wt);
  DS_CHECK_LAUNCH();
  static bool attr = false;
  if (!attr) {
    DS_CUDA(cudaFuncSetAttribute(k_layer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)LG_SMEM_BYTES));
    attr = true;
  }
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    DS_CUDA(cudaGetDevice(&dev));
    DS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  }
  const int grid = std::max(1, std::min(M / 128, sms));
  k_layer_tc<<<grid, LG_THREADS, LG_SMEM_BYTES, st>>>(M, A, wt, bias, Z, out, res, err);
  DS_CHECK_LAUNCH();
}

}  // namespace ds
