// probe.cu — measures the FP64 pipe's issue rate on the current device: the
// denominator of the FP64 roofline that bench.py reports next to the HBM one.
// Independent multiply-add chains (8 per thread, 16 resident blocks per SM)
// keep the pipe saturated; the rate counts one operation per DFMA.
#include <cuda_runtime.h>

#include "../../include/ibmdem.h"

namespace {
constexpr int kChains = 8;
constexpr int kIters = 2048;
__global__ void k_fp64_rate(double* out, double seed) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double a[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) a[c] = seed + 1e-3 * c + 1e-9 * t;
  const double m = 0.9999999, k = 1e-7;
  for (int it = 0; it < kIters; ++it) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) a[c] = fma(a[c], m, k);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += a[c];
  out[t] = s;
}
}  // namespace

extern "C" int ibmdem_measure_fp64_rate(int32_t device, double* gops) {
  if (!gops) return IBMDEM_EINVAL;
  if (cudaSetDevice(device) != cudaSuccess) return IBMDEM_ECUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int blocks = sms * 16, threads = 256;
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return IBMDEM_ENOMEM;
  cudaStream_t s;
  cudaStreamCreate(&s);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fp64_rate<<<blocks, threads, 0, s>>>(out, 1.5);
  float best = 1e30f;
  for (int r = 0; r < 3; ++r) {
    cudaEventRecord(e0, s);
    k_fp64_rate<<<blocks, threads, 0, s>>>(out, 1.5);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  int rc = cudaGetLastError() == cudaSuccess ? IBMDEM_OK : IBMDEM_ECUDA;
  *gops = (double)blocks * threads * kIters * kChains / (best * 1e-3) / 1e9;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  cudaFree(out);
  return rc;
}
