// FP32-mixed path interface (fv_mixed.cu).
#pragma once

#include <vector>

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "fv_kernels.cuh"
#include "fvgpu.h"

namespace fv {

// Device resources the mixed path derives from the mesh at upload time:
// packed per-cell geometry codes, per-level geometry tables, the two FP32
// stage increments, the two FP32 stage-input states, the FP32 gradients of
// viscous runs and the second FP64 state buffer (ping-pong).
struct MixedResources {
  void *buf[11] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  size_t bytes[11] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  size_t cap[11] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};  // allocated bytes (kept across meshes)
  int64_t n = 0;
  int model = 1;           // EOS model the FP32 state layout follows (model 3: density offset)
  int64_t nbricks = 0;     // 8x8x4 brick blocks (structured fast path)
  int64_t nbricks4 = 0;    // 4x4x4 brick blocks
  int64_t ngeneral = 0;    // general blocks
  bool force_general = false;  // FVGPU_FLAG_NO_BRICKS
  // a stage with more than one kind of block runs the 4x4x4 bricks and the
  // general blocks on two more streams, forked from and joined back into the
  // caller's stream
  cudaStream_t side[2] = {nullptr, nullptr};
  cudaEvent_t fork_ev = nullptr, join_ev[2] = {nullptr, nullptr};
  bool ready = false;
  bool snf_valid = false;  // FP32 copy of the current state is up to date
  // kernel family of the prepared mesh: 0 the slope-sharing brick kernel
  // (fv_mixed.cu; meshes of model 1 that are 8x8x4 bricks throughout), 1 the
  // table-driven family (fv_mixed_amr.cu; every other mesh)
  int family = 0;
  int wave = 0;  // resident brick blocks across the GPU (family 0)
  // host copy of the per-level geometry tables (family 1): the general
  // kernel takes them by value, so they sit in the constant bank
  std::vector<unsigned char> geo_host;
};

bool mixed_supported(const Phys &ph, char *why, size_t whylen);
// Builds the mixed-path tables from the host mesh; FVGPU_OK or an error code
// with the reason in `why`.
int mixed_prepare_host(MixedResources &r, const Phys &ph, const fvgpu_mesh_soa *m, char *why, size_t whylen);
void release_mixed(MixedResources &r);
// Forget the prepared mesh but keep the device buffers, streams and events
// for the next one (buffers are reused when large enough).
void reset_mixed(MixedResources &r);
// the second FP64 state buffer (steps write into it; the caller swaps)
double *mixed_alt_state(MixedResources &r);
// exchange the caller's state buffer with the second buffer after a step
void mixed_swap_state(MixedResources &r, void *&state);
// rebuild the FP32 copy of the FP64 state S (after uploads / FP64-path updates)
cudaError_t mixed_refresh_f32(MixedResources &r, const double *S, int neq, LaunchMarks &marks, cudaStream_t st);
// the same, plus the FP32 CFL spectral radius of S max-reduced into *lambda
// (which the caller zeroes)
cudaError_t mixed_refresh_f32_lambda(MixedResources &r, const Phys &ph, const double *S, double *lambda,
                                     LaunchMarks &marks, cudaStream_t st);
namespace amr {
// The table-driven kernel family (fv_mixed_amr.cu): the same entry points.
int mixed_prepare_host(MixedResources &r, const Phys &ph, const fvgpu_mesh_soa *m, char *why, size_t whylen);
void release_mixed(MixedResources &r);
cudaError_t mixed_refresh_f32(MixedResources &r, const double *S, int neq, LaunchMarks &marks, cudaStream_t st);
cudaError_t mixed_refresh_f32_lambda(MixedResources &r, const Phys &ph, const double *S, double *lambda,
                                     LaunchMarks &marks, cudaStream_t st);
cudaError_t enqueue_step_mixed(MixedResources &r, const Phys &ph, const MeshView &m, int scheme, bool cfl_mode,
                               const double *in, double *out, double *dt, double *lambda, const double *cfl,
                               unsigned long long *err, LaunchMarks &marks, cudaStream_t st);
}  // namespace amr

// One RK step from FP64 state `in` to `out` (distinct buffers).
cudaError_t enqueue_step_mixed(MixedResources &r, const Phys &ph, const MeshView &m, int scheme, bool cfl_mode,
                               const double *in, double *out, double *dt, double *lambda, const double *cfl,
                               unsigned long long *err, LaunchMarks &marks, cudaStream_t st);

}  // namespace fv
