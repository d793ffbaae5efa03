// Per-SM throughput of the pipes the roofline figures rest on: FP64 FMA,
// FP32 FMA, MUFU ex2, FP64 exp() and FP64 -> int32 conversion.  Every thread
// runs independent chains of one operation (enough of them to cover the
// pipe's latency); each kernel is timed with CUDA events on its second run.
// out holds grid x block doubles and every kernel writes each thread's entry
// once (the float kernels use the first half of the bytes).
#include <cstdio>

#include <cuda_runtime.h>

#define PR_CHECK(x)                                                           \
  do {                                                                        \
    cudaError_t e_ = (x);                                                     \
    if (e_ != cudaSuccess) {                                                  \
      printf("%s: %s\n", #x, cudaGetErrorString(e_));                         \
      return 1;                                                               \
    }                                                                         \
  } while (0)

__global__ void k_dfma(double* out, int iters, double a, double b) {
  double c[8];
  for (int k = 0; k < 8; ++k) c[k] = threadIdx.x * 1e-9 + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) c[k] = fma(c[k], a, b);
  }
  double s = 0.0;
  for (int k = 0; k < 8; ++k) s += c[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_ffma(float* out, int iters, float a, float b) {
  float c[16];
  for (int k = 0; k < 16; ++k) c[k] = threadIdx.x * 1e-6f + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) c[k] = fmaf(c[k], a, b);
  }
  float s = 0.f;
  for (int k = 0; k < 16; ++k) s += c[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__global__ void k_ex2(float* out, int iters) {
  float c[8];
  for (int k = 0; k < 8; ++k) c[k] = -(threadIdx.x & 7) * 0.01f - k * 0.001f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) c[k] = ex2_approx(c[k]) - 1.0f;
  }
  float s = 0.f;
  for (int k = 0; k < 8; ++k) s += c[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_dexp(double* out, int iters) {
  double c[4];
  for (int k = 0; k < 4; ++k) c[k] = -(threadIdx.x & 7) * 0.01 - k * 0.001;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 4; ++k) c[k] = exp(c[k]) - 1.0;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = c[0] + c[1] + c[2] + c[3];
}

__global__ void k_d2i(double* out, int iters) {
  double c[8];
  for (int k = 0; k < 8; ++k) c[k] = threadIdx.x * 0.37 + k;
  int acc = 0;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      acc += __double2int_rz(c[k]);
      c[k] += 0.5;
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = acc + c[0];
}

int main() {
  cudaDeviceProp p;
  PR_CHECK(cudaGetDeviceProperties(&p, 0));
  int clk_khz = 0;
  PR_CHECK(cudaDeviceGetAttribute(&clk_khz, cudaDevAttrClockRate, 0));
  printf("device %s, %d SMs, clock attribute %d MHz\n", p.name, p.multiProcessorCount,
         clk_khz / 1000);
  const int block = 256, grid = p.multiProcessorCount * 8;
  const size_t n = (size_t)grid * block;
  double* d = nullptr;
  PR_CHECK(cudaMalloc(&d, n * sizeof(double)));
  cudaEvent_t e0, e1;
  PR_CHECK(cudaEventCreate(&e0));
  PR_CHECK(cudaEventCreate(&e1));
  const int it = 4096;
  auto report = [&](const char* name, double ops, float ms) {
    const double per_s = ops / (ms * 1e-3);
    printf("%-6s %8.3f ms  %.3e ops/s  %6.2f per clk per SM (at the attribute clock)\n", name,
           ms, per_s, per_s / (p.multiProcessorCount * (double)clk_khz * 1e3));
  };
  float ms = 0.f;
  for (int rep = 0; rep < 2; ++rep) {
    PR_CHECK(cudaEventRecord(e0));
    k_dfma<<<grid, block>>>(d, it, 0.999, 1e-3);
    PR_CHECK(cudaEventRecord(e1));
    PR_CHECK(cudaEventSynchronize(e1));
    PR_CHECK(cudaEventElapsedTime(&ms, e0, e1));
    if (rep) report("DFMA", (double)n * it * 8, ms);
    PR_CHECK(cudaEventRecord(e0));
    k_ffma<<<grid, block>>>(reinterpret_cast<float*>(d), it * 4, 0.999f, 1e-3f);
    PR_CHECK(cudaEventRecord(e1));
    PR_CHECK(cudaEventSynchronize(e1));
    PR_CHECK(cudaEventElapsedTime(&ms, e0, e1));
    if (rep) report("FFMA", (double)n * it * 4 * 16, ms);
    PR_CHECK(cudaEventRecord(e0));
    k_ex2<<<grid, block>>>(reinterpret_cast<float*>(d), it);
    PR_CHECK(cudaEventRecord(e1));
    PR_CHECK(cudaEventSynchronize(e1));
    PR_CHECK(cudaEventElapsedTime(&ms, e0, e1));
    if (rep) report("EX2", (double)n * it * 8, ms);
    PR_CHECK(cudaEventRecord(e0));
    k_dexp<<<grid, block>>>(d, it / 8);
    PR_CHECK(cudaEventRecord(e1));
    PR_CHECK(cudaEventSynchronize(e1));
    PR_CHECK(cudaEventElapsedTime(&ms, e0, e1));
    if (rep) report("DEXP", (double)n * (it / 8) * 4, ms);
    PR_CHECK(cudaEventRecord(e0));
    k_d2i<<<grid, block>>>(d, it);
    PR_CHECK(cudaEventRecord(e1));
    PR_CHECK(cudaEventSynchronize(e1));
    PR_CHECK(cudaEventElapsedTime(&ms, e0, e1));
    if (rep) report("D2I", (double)n * it * 8, ms);
  }
  PR_CHECK(cudaGetLastError());
  PR_CHECK(cudaDeviceSynchronize());
  PR_CHECK(cudaFree(d));
  return 0;
}
