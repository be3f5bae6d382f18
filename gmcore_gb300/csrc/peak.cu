// Measured fused multiply-add throughput of the current GPU in FP64 and in
// FP32: the peaks against which the two precision forms are placed (the FP64
// form's column sweeps, transcendentals and stencils issue FP64 arithmetic,
// whose rate on GB300 is a small fraction of the FP32 rate; the mixed form's
// stencils are FP32 arithmetic and addressing).  Each thread runs kChains
// independent FMA chains, so the FMA latency is hidden and the pipe's issue
// rate is what is timed; the chains' results are stored so that none of the
// arithmetic is dead.  Timed with CUDA events on a private stream; clocks and
// every other GPU setting are left as they are.
#include <cuda_runtime.h>

#include <algorithm>

#include "gmcore_gpu.h"

namespace {

constexpr int kChains = 8;
constexpr int kIters = 2048;

template <class T>
__global__ void __launch_bounds__(256) k_fma(T *out, T b, T c) {
  T a[kChains];
#pragma unroll
  for (int t = 0; t < kChains; ++t) a[t] = (T)1 + (T)1e-3 * (T)(threadIdx.x + t);
#pragma unroll 16
  for (int it = 0; it < kIters; ++it) {
#pragma unroll
    for (int t = 0; t < kChains; ++t) a[t] = fma(a[t], b, c);
  }
  T s = 0;
#pragma unroll
  for (int t = 0; t < kChains; ++t) s += a[t];
  out[blockIdx.x * (size_t)blockDim.x + threadIdx.x] = s;
}

template <class T>
int fma_peak(double *tflops) {
  if (!tflops) return GMC_EINVAL;
  *tflops = 0;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return GMC_ECUDA;
  }
  const int threads = 256, blocks = sms * 8;
  T *out = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = GMC_OK;
  if (cudaMalloc(&out, (size_t)blocks * threads * sizeof(T)) != cudaSuccess) {
    cudaGetLastError();
    return GMC_ENOMEM;
  }
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
      cudaEventCreate(&e1) != cudaSuccess) {
    rc = GMC_ECUDA;
  }
  // FP32 runs ~64x faster: more repetitions of the loop keep the launch long
  const int reps = sizeof(T) == 4 ? 32 : 1;
  float best = 0;
  for (int rep = 0; rc == GMC_OK && rep < 6; ++rep) {   // the first run warms up; the fastest of the rest counts
    cudaEventRecord(e0, st);
    for (int r = 0; r < reps; ++r) k_fma<T><<<blocks, threads, 0, st>>>(out, (T)0.9999999, (T)1e-7);
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
    const double flops = 2.0 * (double)blocks * threads * kIters * kChains * reps;
    *tflops = flops / (best * 1e-3) / 1e12;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  cudaFree(out);
  cudaGetLastError();
  return rc;
}

}  // namespace

extern "C" int gmc_fp64_fma_peak(double *tflops) { return fma_peak<double>(tflops); }
extern "C" int gmc_fp32_fma_peak(double *tflops) { return fma_peak<float>(tflops); }
