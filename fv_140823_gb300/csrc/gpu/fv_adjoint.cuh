// Launch interface of the FP64 residual adjoint (fv_adjoint.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "fv_physics.cuh"

namespace fv {

// Device arrays of one vector-Jacobian product g = (dR/dU)^T w at state U.
//   U   [5][n]            state the residual is linearised at
//   SF  [6][5][n]         its face values (faceinterp of U; MUSCL only)
//   w   [5][n]            residual weights
//   gL  [6][5][n]         per face: adjoint of the cell's own face value from
//                         its own flux evaluations
//   gR  [6][5][n]         per face with a single neighbour: adjoint of the
//                         neighbour's face value from this cell's evaluation
//   gRh [nhang][4][5]     per sub-face of a 1:4 face: the same for each fine
//                         neighbour
//   gSF [6][5][n]         adjoint of every face value (may alias gL)
//   out [5][n]            result
// viscous runs (ns 1) also:
//   SG   [neq+1][3][n]    gradients of U (gradcalc)
//   gG   [9][n]           bars of each cell's momentum gradients from its own
//                         evaluations
//   gRg  [6][9][n]        per single-neighbour face: the neighbour's gradient bars
//   gRgh [nhang][4][9]    per 1:4 sub-face: the fine neighbour's gradient bars
//   gSG  [9][n]           total gradient bars (may alias gG)
// T is the type of the reverse arithmetic and of the intermediate arrays:
// double for the FP64 path, float for the FP32-mixed path (state, weights,
// gradients and the result stay FP64 arrays).
template <typename T>
struct AdjArgsT {
  const double *U;
  const T *SF;
  const double *w;
  T *gL;
  T *gR;
  T *gRh;
  T *gSF;
  double *out;
  const double *SG;
  T *gG;
  T *gRg;
  T *gRgh;
  T *gSG;
};
using AdjArgs = AdjArgsT<double>;

// true when the adjoint implements the configuration (model 1);
// otherwise writes the reason
bool adjoint_supported(const Phys &ph, char *why, size_t whylen);

// the gather passes of g = (dR/dU)^T w (faceinterp of U, and gradcalc of U
// for ns 1, must precede)
void launch_adjoint(const Phys &ph, const MeshView &m, const AdjArgs &a, cudaStream_t st);
// the same passes in FP32 (face values from launch_faceinterp_f32, FP64
// gradcalc for ns 1)
void launch_adjoint_f32(const Phys &ph, const MeshView &m, const AdjArgsT<float> &a, cudaStream_t st);
// FP32 face values of the FP64 state U for the FP32 passes
void launch_faceinterp_f32(const Phys &ph, const MeshView &m, const double *U, float *SF, cudaStream_t st);

// w = coef * dt / vol * g
void launch_adj_scale(const MeshView &m, const double *g, const double *dt, double coef, double *w,
                      cudaStream_t st);

// y = alpha * x + beta * y over count doubles
void launch_axpby(int64_t count, double alpha, const double *x, double beta, double *y, cudaStream_t st);

}  // namespace fv
