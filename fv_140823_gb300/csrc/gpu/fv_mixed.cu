// FP32-mixed path (placeholder interface until the kernels land).
#include <cstdio>

#include "fv_mixed.cuh"

namespace fv {

bool mixed_supported(const Phys &ph, char *why, size_t whylen) {
  (void)ph;
  snprintf(why, whylen, "the mixed-precision path is not available in this build");
  return false;
}

cudaError_t prepare_mixed(MixedResources &r, const Phys &, const MeshView &, const int32_t *, cudaStream_t) {
  r.ready = false;
  return cudaErrorNotSupported;
}

void release_mixed(MixedResources &r) {
  for (int i = 0; i < 8; ++i) {
    if (r.buf[i]) cudaFree(r.buf[i]);
    r.buf[i] = nullptr;
    r.bytes[i] = 0;
  }
  r.ready = false;
}

cudaError_t enqueue_step_mixed(MixedResources &, const Phys &, const MeshView &, int, bool, double *, double *,
                               double *, double *, const double *, unsigned long long *, LaunchMarks &,
                               cudaStream_t) {
  return cudaErrorNotSupported;
}

}  // namespace fv
