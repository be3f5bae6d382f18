// Measured FP64 fused multiply-add throughput of the current GPU: the peak
// against which the FP64 form's kernels are placed (its column sweeps,
// transcendentals and stencils issue FP64 arithmetic, whose rate on GB300 is a
// small fraction of the FP32 rate).  Each thread runs kChains independent
// FMA chains, so the FMA latency is hidden and the pipe's issue rate is what
// is timed; the chains' results are stored so that none of the arithmetic is
// dead.  Timed with CUDA events on a private stream; clocks and every other
// GPU setting are left as they are.
#include <cuda_runtime.h>

#include <algorithm>

#include "gmcore_gpu.h"

namespace {

constexpr int kChains = 8;
constexpr int kIters = 2048;

__global__ void __launch_bounds__(256) k_fp64_fma(double *out, double b, double c) {
  double a[kChains];
#pragma unroll
  for (int t = 0; t < kChains; ++t) a[t] = 1.0 + 1e-3 * (threadIdx.x + t);
  for (int it = 0; it < kIters; ++it) {
#pragma unroll
    for (int t = 0; t < kChains; ++t) a[t] = fma(a[t], b, c);
  }
  double s = 0;
#pragma unroll
  for (int t = 0; t < kChains; ++t) s += a[t];
  out[blockIdx.x * (size_t)blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" int gmc_fp64_fma_peak(double *tflops) {
  if (!tflops) return GMC_EINVAL;
  *tflops = 0;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return GMC_ECUDA;
  }
  const int threads = 256, blocks = sms * 8;
  double *out = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = GMC_OK;
  if (cudaMalloc(&out, (size_t)blocks * threads * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    return GMC_ENOMEM;
  }
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
      cudaEventCreate(&e1) != cudaSuccess) {
    rc = GMC_ECUDA;
  }
  float best = 0;
  for (int rep = 0; rc == GMC_OK && rep < 6; ++rep) {   // the first run warms up; the fastest of the rest counts
    cudaEventRecord(e0, st);
    k_fp64_fma<<<blocks, threads, 0, st>>>(out, 0.9999999, 1e-7);
    cudaEventRecord(e1, st);
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      rc = GMC_ECUDA;
      break;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && (best == 0 || ms < best)) best = ms;
  }
  if (rc == GMC_OK && cudaGetLastError() != cudaSuccess) rc = GMC_ECUDA;
  if (rc == GMC_OK && best > 0) {
    const double flops = 2.0 * (double)blocks * threads * kIters * kChains;
    *tflops = flops / (best * 1e-3) / 1e12;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  cudaFree(out);
  cudaGetLastError();
  return rc;
}
