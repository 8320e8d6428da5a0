// Kernel launch interface shared by the C-ABI layer (fv_api.cu) and the
// kernel translation units (fv_fp64.cu, fv_mixed.cu, fv_adjoint.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "fv_physics.cuh"

namespace fv {

// Optional per-launch event marks (fvgpu_profile_step).  mark(kind) is called
// right before each kernel launch; when active it records an event on the
// stream, so the time between consecutive marks is the kernel's device time.
struct LaunchMarks {
  bool active = false;
  cudaStream_t stream = nullptr;
  cudaEvent_t *events = nullptr;
  int *kinds = nullptr;
  int capacity = 0;
  int used = 0;
  int counts[FVGPU_NKINDS] = {0, 0, 0, 0, 0, 0, 0, 0};
  void mark(int kind) {
    if (kind >= 0 && kind < FVGPU_NKINDS) counts[kind]++;
    if (!active || used >= capacity) return;
    kinds[used] = kind;
    cudaEventRecord(events[used], stream);
    ++used;
  }
};

// Arguments of the residual kernel.
//   irk == 0 : write the residual to R (RHS(run)).
//   irk >= 1 : fused RK(irk) stage, S_out <- RK update of U (in place when
//              S_out == U, allowed for MUSCL where neighbours are read from
//              SF only); irk == 1 also writes SN <- U (RK(0)).  R, when not
//              null, receives the residual as well.  lambda, when not null,
//              receives the max CFL spectral radius of the updated state.
struct ResidualArgs {
  const double *U;
  const double *SF;
  const double *SG;
  double *R;
  double *S_out;
  double *SN;
  const double *dt;
  double *lambda;
  const int32_t *inner;
  int inner_outer;
  int irk;
  unsigned long long *err;
};

// FP64 path (fv_fp64.cu)
void launch_faceinterp_fp64(const Phys &ph, const MeshView &m, const double *U, double *SF, cudaStream_t st);
void launch_gradcalc_fp64(const Phys &ph, const MeshView &m, const double *U, double *SG,
                          unsigned long long *err, cudaStream_t st);
void launch_residual_fp64(const Phys &ph, const MeshView &m, const ResidualArgs &a, cudaStream_t st);
void launch_rk_fp64(int irk, const Phys &ph, const MeshView &m, double *S, double *SN, const double *R,
                    const double *dt, double *lambda, cudaStream_t st);
void launch_lambda_fp64(const Phys &ph, const MeshView &m, const double *U, double *lambda, cudaStream_t st);

// Reductions and small helpers (fv_api.cu)
void launch_dt_from_lambda(const double *lambda_in, double *lambda_reset, const double *cfl, double *dt,
                           unsigned long long *err, cudaStream_t st);

}  // namespace fv
