// FP32 issue-rate probe: the denominator of the search kernels' roofline.
//
// The semblance search is bound by FP32 arithmetic and shared-memory loads, not by
// HBM or the tensor cores, so its roofline needs the GPU's FP32 fused-multiply-add
// throughput, which this probe measures: every thread runs 8 independent FMA
// chains, the grid fills every SM several times over, and the rate is 2 flops per
// FMA over the CUDA-event time.
#include <cuda_runtime.h>

#include "common.h"
#include "semb_kernels.cuh"

namespace {

__global__ void __launch_bounds__(256) k_fma_chains(int iters, float seed, float* out) {
  float a0 = seed + threadIdx.x, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f;
  float a4 = a0 + 4.f, a5 = a0 + 5.f, a6 = a0 + 6.f, a7 = a0 + 7.f;
  const float m = 0.999999f, c = 1e-7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      a0 = fmaf(a0, m, c); a1 = fmaf(a1, m, c); a2 = fmaf(a2, m, c); a3 = fmaf(a3, m, c);
      a4 = fmaf(a4, m, c); a5 = fmaf(a5, m, c); a6 = fmaf(a6, m, c); a7 = fmaf(a7, m, c);
    }
  }
  const float s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
  if (s == 12345.678f) out[0] = s;   // keeps the chains live
}

}  // namespace

extern "C" int semb_probe_fp32(int32_t device, double* tflops) {
  if (!tflops) return semb::fail(SEMB_E_ARG, "null argument");
  *tflops = 0.0;
  if (device < 0 || device >= semb_device_count()) return semb::fail(SEMB_E_NODEV, "device %d not available", device);
  SEMB_CUDA(cudaSetDevice(device));
  cudaDeviceProp prop;
  SEMB_CUDA(cudaGetDeviceProperties(&prop, device));
  const int blocks = prop.multiProcessorCount * 8, threads = 256, iters = 4096;
  float* out = nullptr;
  SEMB_CUDA(cudaMalloc(&out, sizeof(float)));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fma_chains<<<blocks, threads>>>(64, 1.f, out);   // warm-up
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    k_fma_chains<<<blocks, threads>>>(iters, 1.f + rep, out);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    best = ms < best ? ms : best;
  }
  cudaError_t e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  SEMB_CUDA(e);
  const double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
  *tflops = flops / (best * 1e-3) / 1e12;
  return SEMB_OK;
}

namespace {

// One CTA waits on a barrier phase that nothing completes, through the same
// bounded wait the search kernels use for their bulk copies, and reports whether
// the wait gave up (1) or completed (0).
__global__ void k_wait_selftest(uint64_t limit_ns, int* timed_out) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    semb::mbar_init(&bar, 1);
    semb::fence_mbar_init();
  }
  __syncthreads();
  const bool ok = semb::wait_bar(&bar, 0, limit_ns);
  if (threadIdx.x == 0) *timed_out = ok ? 0 : 1;
}

}  // namespace

extern "C" int semb_selftest_wait(int32_t device, int64_t limit_us, int32_t* timed_out) {
  if (!timed_out || limit_us <= 0 || limit_us > 10000000) return semb::fail(SEMB_E_ARG, "bad argument");
  if (device < 0 || device >= semb_device_count()) return semb::fail(SEMB_E_NODEV, "device %d not available", device);
  SEMB_CUDA(cudaSetDevice(device));
  int* d = nullptr;
  SEMB_CUDA(cudaMalloc(&d, sizeof(int)));
  k_wait_selftest<<<1, 32>>>((uint64_t)limit_us * 1000ull, d);
  cudaError_t e = cudaGetLastError();
  int h = -1;
  if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d);
  SEMB_CUDA(e);
  *timed_out = h;
  return SEMB_OK;
}
