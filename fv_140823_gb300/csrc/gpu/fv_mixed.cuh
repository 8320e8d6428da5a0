// FP32-mixed path interface (fv_mixed.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "fv_kernels.cuh"

namespace fv {

// Device resources the mixed path derives from the mesh at upload time.
struct MixedResources {
  void *buf[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  size_t bytes[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  bool ready = false;
};

bool mixed_supported(const Phys &ph, char *why, size_t whylen);
cudaError_t prepare_mixed(MixedResources &r, const Phys &ph, const MeshView &m, const int32_t *level,
                          cudaStream_t st);
void release_mixed(MixedResources &r);
cudaError_t enqueue_step_mixed(MixedResources &r, const Phys &ph, const MeshView &m, int scheme, bool cfl_mode,
                               double *S, double *SN, double *dt, double *lambda, const double *cfl,
                               unsigned long long *err, LaunchMarks &marks, cudaStream_t st);

}  // namespace fv
