// Pipe-throughput calibration for bench.py's rooflines: how many exact-kernel
// pairs per second the FP32 FMA and MUFU pipes of this GPU sustain when they
// run together in the pair kernel's instruction mix, measured in the same run
// as the kernel it bounds.
//
// Per pair the FP32 pair kernels issue 1 MUFU ex2 and 4 FP32 FMA lanes (two
// f32x2 FFMA2: three for the exponent of two pairs, one for the accumulation
// of two).  The pipes' separate rates (ex2 and FFMA2 alone, also printed)
// suggest 32 pairs per clock per SM, but together they do not reach it; the
// mixed loop here (independent chains per thread, no memory traffic) is the
// ceiling that instruction mix can reach, taken as the best over several
// occupancies and chain counts.
//
// Build: nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o <exe> bench_pipes.cu
// Output: one JSON line {"ex2_per_s", "ffma_lanes_per_s", "mix_pairs_per_s",
// "mix_best": {"chains", "warps_per_sm"}, "sms", "clock_attribute_mhz"}.
#include <cstdio>

#include <cuda_runtime.h>

namespace {

__device__ __forceinline__ float ex2f(float x) {
  float y;
  asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

constexpr int ITERS = 4000;  // loop trips per thread, passed at run time

// MUFU alone: 8 independent ex2 chains, values kept in [-1, 0).
__global__ void k_ex2(float* out, int iters) {
  float c[8];
  for (int k = 0; k < 8; ++k) c[k] = -0.001f * (threadIdx.x + k);
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int k = 0; k < 8; ++k) c[k] = -ex2f(c[k]);
  float s = 0.f;
  for (int k = 0; k < 8; ++k) s += c[k];
  if (s == 12345.f) out[0] = s;  // keeps the chains live
}

// FFMA2 alone: 8 independent chains.
__global__ void k_ffma2(float* out, int iters) {
  float2 c[8];
  const float2 a = make_float2(0.999f, 0.998f), b = make_float2(1e-3f, 2e-3f);
  for (int k = 0; k < 8; ++k) c[k] = make_float2(threadIdx.x * 1e-3f + k, (float)k);
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int k = 0; k < 8; ++k) c[k] = __ffma2_rn(c[k], a, b);
  float s = 0.f;
  for (int k = 0; k < 8; ++k) s += c[k].x + c[k].y;
  if (s == 12345.f) out[0] = s;
}

// The pair kernel's mix, NC independent chains of two pairs each:
// t = 3 FFMA2 (exponent), e = 2 ex2, acc = FFMA2 (accumulation).
template <int NC>
__global__ void k_mix(float* out, int iters) {
  float2 acc[NC], x[NC];
  const float2 cx = make_float2(-0.01f, -0.01f), cy = make_float2(0.02f, 0.02f);
  const float2 cz = make_float2(-0.03f, -0.03f), cw = make_float2(-1.0f, -1.0f);
  const float2 u = make_float2(1e-6f, 1e-6f);
  for (int k = 0; k < NC; ++k) {
    acc[k] = make_float2(0.f, 0.f);
    x[k] = make_float2(threadIdx.x * 1e-4f + k, k * 0.5f);
  }
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      float2 t = __ffma2_rn(x[k], cx, cw);
      t = __ffma2_rn(acc[k], cy, t);
      t = __ffma2_rn(x[k], cz, t);
      const float2 e = make_float2(ex2f(t.x), ex2f(t.y));
      acc[k] = __ffma2_rn(e, u, acc[k]);
    }
  float s = 0.f;
  for (int k = 0; k < NC; ++k) s += acc[k].x + acc[k].y;
  if (s == 12345.f) out[0] = s;
}

}  // namespace

int main() {
  int sms = 0, clk_khz = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0) != cudaSuccess) return 1;
  cudaDeviceGetAttribute(&clk_khz, cudaDevAttrClockRate, 0);
  float* d = nullptr;
  if (cudaMalloc(&d, 16) != cudaSuccess) return 1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // best of three timed launches after one warm-up
  auto rate = [&](void (*k)(float*, int), int ctas_per_sm, int block, double ops_per_thread) {
    const int grid = sms * ctas_per_sm;
    double best = 0.0;
    for (int rep = 0; rep < 4; ++rep) {
      cudaEventRecord(e0);
      k<<<grid, block>>>(d, ITERS);  // a run-time count: the loops stay loops
      cudaEventRecord(e1);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      const double r = (double)grid * block * ops_per_thread / (ms * 1e-3);
      if (rep > 0 && r > best) best = r;
    }
    return best;
  };
  const double ex2 = rate(k_ex2, 8, 256, 8.0 * ITERS);
  const double ffma = rate(k_ffma2, 8, 256, 16.0 * ITERS);
  double mix = 0.0;
  int best_nc = 0, best_warps = 0;
  for (int per_sm : {5, 8, 16}) {
    const double r1 = rate(k_mix<1>, per_sm, 128, 2.0 * ITERS);
    const double r2 = rate(k_mix<2>, per_sm, 128, 4.0 * ITERS);
    const double r8 = rate(k_mix<8>, per_sm, 128, 16.0 * ITERS);
    const double rs[3] = {r1, r2, r8};
    const int ncs[3] = {1, 2, 8};
    for (int q = 0; q < 3; ++q)
      if (rs[q] > mix) {
        mix = rs[q];
        best_nc = ncs[q];
        best_warps = per_sm * 4;
      }
  }
  const cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) {
    fprintf(stderr, "bench_pipes: %s\n", cudaGetErrorString(err));
    return 1;
  }
  printf("{\"ex2_per_s\": %.6e, \"ffma_lanes_per_s\": %.6e, \"mix_pairs_per_s\": %.6e, "
         "\"mix_best\": {\"chains\": %d, \"warps_per_sm\": %d}, \"sms\": %d, "
         "\"clock_attribute_mhz\": %d}\n",
         ex2, ffma, mix, best_nc, best_warps, sms, clk_khz / 1000);
  cudaFree(d);
  return 0;
}
