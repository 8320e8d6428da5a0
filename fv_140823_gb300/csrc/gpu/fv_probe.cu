// fvbuild: -fmad=false
//
// Measured FP64 arithmetic peak (the denominator of the FP64 path's
// roofline): separate double-precision adds and multiplies, as the FP64
// path issues them (-fmad=false), from registers, on every SM.
#include <cuda_runtime.h>

#include "fvgpu.h"

namespace {

constexpr int kIters = 2048;
constexpr int kChains = 8;

__global__ void __launch_bounds__(256) k_fp64_rate(double x, double y, double *out) {
  double a[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) a[k] = 1.0 + 1e-3 * double(threadIdx.x + k);
#pragma unroll 4
  for (int i = 0; i < kIters; ++i) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = __dadd_rn(__dmul_rn(a[k], x), y);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += a[k];
  if (s == 12345.678) out[0] = s;  // keeps the chains live; never true for these inputs
}

}  // namespace

extern "C" int fvgpu_measure_fp64(int device, double *gops) {
  if (!gops) return FVGPU_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return FVGPU_ERR_NODEVICE;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  double *out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return FVGPU_ERR_NOMEM;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const unsigned blocks = unsigned(sms * 8), threads = 256;
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {  // the first launch is a warm-up
    cudaEventRecord(e0);
    k_fp64_rate<<<blocks, threads>>>(0.999999, 1e-7, out);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return FVGPU_ERR_CUDA;
  const double ops = double(blocks) * threads * kIters * kChains * 2.0;
  *gops = ops / (double(best) * 1e-3) / 1e9;
  return FVGPU_OK;
}
