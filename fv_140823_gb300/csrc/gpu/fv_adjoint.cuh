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
struct AdjArgs {
  const double *U;
  const double *SF;
  const double *w;
  double *gL;
  double *gR;
  double *gRh;
  double *gSF;
  double *out;
};

// true when the adjoint implements the configuration (model 1, inviscid);
// otherwise writes the reason
bool adjoint_supported(const Phys &ph, char *why, size_t whylen);

// the three gather passes of g = (dR/dU)^T w (faceinterp of U must precede)
void launch_adjoint(const Phys &ph, const MeshView &m, const AdjArgs &a, cudaStream_t st);

// w = coef * dt / vol * g
void launch_adj_scale(const MeshView &m, const double *g, const double *dt, double coef, double *w,
                      cudaStream_t st);

// y = alpha * x + beta * y over count doubles
void launch_axpby(int64_t count, double alpha, const double *x, double beta, double *y, cudaStream_t st);

}  // namespace fv
