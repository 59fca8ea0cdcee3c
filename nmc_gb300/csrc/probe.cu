// probe.cu - measured issue-rate denominators for the roofline of the
// transport kernels (which are FP32/INT-issue and SFU bound, not HBM or
// tensor bound): FP32 FMA lanes/s and MUFU (ex2) lanes/s on this GPU, timed
// with CUDA events.  Measurement support; no counterpart in the reference.
#include <cuda_runtime.h>

#include "engine.h"
#include "nmc_abi.h"

namespace {

constexpr int kChains = 8;

__global__ void __launch_bounds__(256) ffma_probe(float* out, int iters, float a, float b) {
  float x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = threadIdx.x * 1e-3f + c;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = fmaf(x[c], a, b);
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  if (s == 1234.5f) out[threadIdx.x] = s;  // keeps the chains live
}

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__global__ void __launch_bounds__(256) mufu_probe(float* out, int iters) {
  float x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = -1e-3f * (threadIdx.x + c);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = ex2_approx(x[c]) - 1.0f;
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  if (s == 1234.5f) out[threadIdx.x] = s;
}

}  // namespace

extern "C" nmc_status nmc_probe_issue_peaks(int32_t device, double* ffma_lanes_per_s,
                                            double* mufu_lanes_per_s) {
  if (!ffma_lanes_per_s || !mufu_lanes_per_s) return NMC_EINVAL;
  nmc::DeviceScope dev(device);
  if (!dev.ok) return NMC_EDEVICE;
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
  float* out = nullptr;
  if (cudaMalloc(&out, 256 * sizeof(float)) != cudaSuccess) return NMC_EDEVICE;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const int block = 256, grid = nsm * 8, iters = 4096;
  double best_f = 0, best_m = 0;
  for (int rep = 0; rep < 3; ++rep) {
    float ms = 0.f;
    cudaEventRecord(a);
    ffma_probe<<<grid, block>>>(out, iters, 0.9999f, 1e-4f);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    cudaEventElapsedTime(&ms, a, b);
    const double f = (double)grid * block * iters * kChains / (ms * 1e-3);
    if (rep && f > best_f) best_f = f;
    cudaEventRecord(a);
    mufu_probe<<<grid, block>>>(out, iters / 4);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    cudaEventElapsedTime(&ms, a, b);
    const double m = (double)grid * block * (iters / 4) * kChains / (ms * 1e-3);
    if (rep && m > best_m) best_m = m;
  }
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  if (err != cudaSuccess) return NMC_EDEVICE;
  *ffma_lanes_per_s = best_f;
  *mufu_lanes_per_s = best_m;
  return NMC_OK;
}
