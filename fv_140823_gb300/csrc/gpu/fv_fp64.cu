// fvbuild: -fmad=false
//
// FP64 path: the reference's residual evaluation and RK stage update, one
// thread per cell, every face evaluated from both of its sides in the
// reference's order (residual_faces_AMR.c walks each leaf's faces and
// sub-faces and computes each face flux from the leaf's own side).  Compiled
// with -fmad=false: with no fused multiply-adds and IEEE division / square
// root, each cell's results are bit-identical to the reference's C code.
//
// GB300 note: FP64 throughput on this part is a small fraction of FP32, so
// these kernels are bound by the FP64 pipe, not by HBM; the FP32-mixed path
// (fv_mixed.cu) is the bandwidth-oriented one.
#include "fv_kernels.cuh"

namespace fv {

namespace {

constexpr int kBlock = 128;

__device__ __forceinline__ void load_state(const double *__restrict__ U, int neq, int64_t n, int64_t c,
                                           double q[kNeqMax]) {
#pragma unroll
  for (int v = 0; v < kNeqMax; ++v) q[v] = v < neq ? U[v * n + c] : 0.0;
}

// deltavalues.c:3-26 with facevalues_MUSCL.c:3-56: neighbour (mean of the
// four fine neighbours of a 1:4 face, or boundary ghost) minus own.
__device__ __forceinline__ void delta_values(const Phys &ph, const MeshView &m, const double *__restrict__ U,
                                             int64_t c, int f, const double own[kNeqMax],
                                             double delta[kNeqMax]) {
  const int neq = ph.neq;
  const int64_t n = m.n;
  const int32_t code = m.nbr[f * n + c];
  double nb[kNeqMax];
  if (code >= 0) {
    load_state(U, neq, n, code, nb);
  } else if (is_hanging(code)) {
    const int32_t *k = m.hang_nbr + 4 * hang_index(code);
#pragma unroll
    for (int v = 0; v < kNeqMax; ++v) nb[v] = 0.0;
    for (int s = 0; s < 4; ++s) {
      const int64_t ks = k[s];
#pragma unroll
      for (int v = 0; v < kNeqMax; ++v)
        if (v < neq) nb[v] += U[v * n + ks] / ((double)4);
    }
  } else {
    const int bc = -1 - code;
    FaceState<double> g;
#pragma unroll
    for (int v = 0; v < kNeqMax; ++v) g.vec[v] = own[v];
    if (bc == 1 || bc == 3 || bc == 4) {
      face_state(ph, own, false, g);
      apply_bc(ph, bc, f, g);
    }
#pragma unroll
    for (int v = 0; v < kNeqMax; ++v) nb[v] = g.vec[v];
  }
#pragma unroll
  for (int v = 0; v < kNeqMax; ++v) delta[v] = nb[v] - own[v];
}

// faceinterp.c:21-61 -> reconctruct_V3.c:3-57 (minmod, iprimtv = 0).
__global__ void __launch_bounds__(kBlock) k_faceinterp(Phys ph, MeshView m, const double *__restrict__ U,
                                                       double *__restrict__ SF) {
  const int64_t c = int64_t(blockIdx.x) * kBlock + threadIdx.x;
  if (c >= m.n) return;
  const int neq = ph.neq;
  const int64_t n = m.n;
  double own[kNeqMax];
  load_state(U, neq, n, c, own);
  double delta[6][kNeqMax];
#pragma unroll
  for (int f = 0; f < 6; ++f) delta_values(ph, m, U, c, f, own, delta[f]);
#pragma unroll
  for (int f = 0; f < 6; ++f) {
    const int fo = opp_face(f);
    const double dist_p1_cf = m.dcf[f * n + c];
    const double dist_p1_cc = m.dcc[f * n + c];
    const double dist_m1_cc = m.dcc[fo * n + c];
    const bool bcf = is_boundary(m.nbr[f * n + c]);
#pragma unroll
    for (int iv = 0; iv < kNeqMax; ++iv) {
      if (iv >= neq) break;
      const double d0 = delta[f][iv], d1 = delta[fo][iv];
      double grad = 0.0;
      if (!bcf) {
        if (fabs(d0) > 1e-10) {  // pow(10.0,-10.0) == 1e-10
          const double product = (-d1 / dist_m1_cc) * (d0 / dist_p1_cc);
          if (product > 0.0) {
            if (fabs(-d1 / dist_m1_cc) > fabs(d0 / dist_p1_cc))
              grad = d0 / dist_p1_cc;
            else
              grad = -d1 / dist_m1_cc;
          } else {
            grad = 0.0;
          }
        }
      }
      SF[(f * neq + iv) * n + c] = own[iv] + dist_p1_cf * grad;
    }
  }
}

// gradcalc.c:9-47: Green-Gauss gradients of the conservative variables and of
// the pressure, first-order face values (facevalues.c).
__global__ void __launch_bounds__(kBlock) k_gradcalc(Phys ph, MeshView m, const double *__restrict__ U,
                                                     double *__restrict__ SG, unsigned long long *err) {
  const int64_t c = int64_t(blockIdx.x) * kBlock + threadIdx.x;
  if (c >= m.n) return;
  const int neq = ph.neq;
  const int64_t n = m.n;
  double own[kNeqMax];
  load_state(U, neq, n, c, own);
  const double Vol = m.vol[c];
  double g[kNeqMax + 1][3];
#pragma unroll
  for (int iv = 0; iv <= kNeqMax; ++iv) g[iv][0] = g[iv][1] = g[iv][2] = 0.0;
  FaceState<double> s;
  bool ok = face_state(ph, own, false, s);
#pragma unroll
  for (int f = 0; f < 6; ++f) {
    const int32_t code = m.nbr[f * n + c];
    const double nx = ph.frames[9 * f], ny = ph.frames[9 * f + 1], nz = ph.frames[9 * f + 2];
    const int nsub = is_hanging(code) ? 4 : 1;
    for (int ing = 0; ing < nsub; ++ing) {
      FaceState<double> s1;
      double A;
      if (code >= 0) {
        double q[kNeqMax];
        load_state(U, neq, n, code, q);
        ok &= face_state(ph, q, false, s1);
        A = m.area[f * n + c];
      } else if (is_hanging(code)) {
        const int64_t r = hang_index(code);
        double q[kNeqMax];
        load_state(U, neq, n, m.hang_nbr[4 * r + ing], q);
        ok &= face_state(ph, q, false, s1);
        A = m.hang_area[4 * r + ing];
      } else {
        s1 = s;
        apply_bc(ph, -1 - code, f, s1);
        A = m.area[f * n + c];
      }
#pragma unroll
      for (int iv = 0; iv < kNeqMax; ++iv) {
        if (iv >= neq) break;
        g[iv][0] += 0.5 * (s1.vec[iv] + s.vec[iv]) * nx * A / Vol;
        g[iv][1] += 0.5 * (s1.vec[iv] + s.vec[iv]) * ny * A / Vol;
        g[iv][2] += 0.5 * (s1.vec[iv] + s.vec[iv]) * nz * A / Vol;
      }
      g[neq][0] += 0.5 * (s1.p + s.p) * nx * A / Vol;
      g[neq][1] += 0.5 * (s1.p + s.p) * ny * A / Vol;
      g[neq][2] += 0.5 * (s1.p + s.p) * nz * A / Vol;
    }
  }
  if (!ok) raise_error(err, kErrEos, c);
  for (int iv = 0; iv <= neq; ++iv)
#pragma unroll
    for (int d = 0; d < 3; ++d) SG[(iv * 3 + d) * n + c] = g[iv][d];
}

__device__ __forceinline__ void load_grad9(const double *__restrict__ SG, int64_t n, int64_t c, double g[9]) {
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int d = 0; d < 3; ++d) g[a * 3 + d] = SG[((1 + a) * 3 + d) * n + c];
}

// Per-cell CFL spectral radius (no reference code; definition in fvgpu.h).
__device__ __forceinline__ double cell_lambda(const Phys &ph, const MeshView &m, int64_t c,
                                              const double q[kNeqMax]) {
  FaceState<double> s;
  face_state(ph, q, false, s);
  double acc = 0.0;
  const int64_t n = m.n;
#pragma unroll
  for (int f = 0; f < 6; ++f) {
    const double *fr = ph.frames + 9 * f;
    const double un = fabs(s.u * fr[0] + s.v * fr[1] + s.w * fr[2]);
    const int32_t code = m.nbr[f * n + c];
    if (is_hanging(code)) {
      const int64_t r = hang_index(code);
      for (int k = 0; k < 4; ++k) acc += m.hang_area[4 * r + k] * (un + s.c);
    } else {
      acc += m.area[f * n + c] * (un + s.c);
    }
  }
  return acc / (2.0 * m.vol[c]);
}

// Block max of a non-negative double, folded into *out with an integer
// atomicMax on its bit pattern (order-independent, hence deterministic).  A
// NaN lambda is folded as +Inf-or-larger bits, which the dt kernel rejects.
__device__ __forceinline__ void block_max_lambda(double lam, double *out) {
  __shared__ double red[kBlock / 32];
  for (int o = 16; o > 0; o >>= 1) lam = fmax(lam, __shfl_xor_sync(0xffffffffu, lam, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = lam;
  __syncthreads();
  if (threadIdx.x == 0) {
    double mx = red[0];
    for (int w = 1; w < kBlock / 32; ++w) mx = fmax(mx, red[w]);
    if (mx > 0.0 || isnan(mx))
      atomicMax((unsigned long long *)out, (unsigned long long)__double_as_longlong(mx));
  }
}

// RK.c:16-47 stage formulas.
__device__ __forceinline__ double rk_update(int irk, double S, double SN, double R, double dt, double Vol) {
  switch (irk) {
    case 1:
      return SN + dt * (1.0 / Vol) * R;
    case 2:
      return (3.0 / 4.0) * SN + (1.0 / 4.0) * S + (1.0 / 4.0) * dt * R / Vol;
    case 3:
      return (1.0 / 3.0) * SN + (2.0 / 3.0) * S + (2.0 / 3.0) * dt * R / Vol;
    case 4:
      return (1.0 / 2.0) * SN + (1.0 / 2.0) * S + (1.0 / 2.0) * dt * R / Vol;
    default:
      return S;
  }
}

// residual_faces_AMR.c:10-202 for one cell; optional fused RK stage.
template <bool MUSCL, bool NS>
__global__ void __launch_bounds__(kBlock) k_residual(Phys ph, MeshView m, ResidualArgs a) {
  const int64_t c = int64_t(blockIdx.x) * kBlock + threadIdx.x;
  const bool active = c < m.n && (a.inner == nullptr || a.inner[c] == a.inner_outer);
  double lam = 0.0;
  if (active) {
    const int neq = ph.neq;
    const int64_t n = m.n;
    double rhs[kNeqMax], FV[kNeqMax][3];
#pragma unroll
    for (int iv = 0; iv < kNeqMax; ++iv) {
      rhs[iv] = 0.0;
      FV[iv][0] = FV[iv][1] = FV[iv][2] = 0.0;
    }
    double g9own[9];
    if (NS) load_grad9(a.SG, n, c, g9own);
    bool ok_eos = true, ok_region = true;
#pragma unroll 1
    for (int f = 0; f < 6; ++f) {
      const int32_t code = m.nbr[f * n + c];
      const double *fr = ph.frames + 9 * f;
      const bool boundary = is_boundary(code);
      const int Nneig = is_hanging(code) ? 4 : 1;
      double flux_face[kNeqMax];
#pragma unroll
      for (int iv = 0; iv < kNeqMax; ++iv) flux_face[iv] = 0.0;
      double qown[kNeqMax];
#pragma unroll
      for (int v = 0; v < kNeqMax; ++v)
        qown[v] = v < neq ? (MUSCL ? a.SF[(f * neq + v) * n + c] : a.U[v * n + c]) : 0.0;
      FaceState<double> s;
      ok_eos &= face_state(ph, qown, MUSCL, s);
      if (NS)
#pragma unroll
        for (int k = 0; k < 9; ++k) s.g[k] = g9own[k];
      const int nf = m.nbr_face[f * n + c];
#pragma unroll 1
      for (int ineig = 0; ineig < Nneig; ++ineig) {
        FaceState<double> s1;
        double A;
        if (boundary) {
          s1 = s;
          apply_bc(ph, -1 - code, f, s1);
          A = m.area[f * n + c];
        } else {
          int64_t k;
          if (code >= 0) {
            k = code;
            A = m.area[f * n + c];
          } else {
            const int64_t r = hang_index(code);
            k = m.hang_nbr[4 * r + ineig];
            A = m.hang_area[4 * r + ineig];
          }
          double q[kNeqMax];
#pragma unroll
          for (int v = 0; v < kNeqMax; ++v)
            q[v] = v < neq ? (MUSCL ? a.SF[(nf * neq + v) * n + k] : a.U[v * n + k]) : 0.0;
          ok_eos &= face_state(ph, q, MUSCL, s1);
          if (NS) load_grad9(a.SG, n, k, s1.g);
        }
        if (NS) flux_viscous(ph, s, s1, FV);
        double F[kNeqMax][3], FH[kNeqMax];
        ok_region &= hllc(ph, f, boundary ? -1 - code : 0, s, s1, F, FH);
#pragma unroll
        for (int iv = 0; iv < kNeqMax; ++iv) {
          if (iv >= neq) break;
          if (NS)
            flux_face[iv] += -(A) * (((F[iv][0] - FV[iv][0]) * fr[0] + (F[iv][1] - FV[iv][1]) * fr[1] +
                                      (F[iv][2] - FV[iv][2]) * fr[2]) +
                                     FH[iv]);
          else  // (F - 0.0) == F for every F, so the zero viscous terms drop out exactly
            flux_face[iv] += -(A) * ((F[iv][0] * fr[0] + F[iv][1] * fr[1] + F[iv][2] * fr[2]) + FH[iv]);
        }
      }
#pragma unroll
      for (int iv = 0; iv < kNeqMax; ++iv) rhs[iv] += flux_face[iv];
    }
    bool finite = true;
#pragma unroll
    for (int iv = 0; iv < kNeqMax; ++iv)
      if (iv < neq && isnan(rhs[iv])) finite = false;
    if (!ok_eos) raise_error(a.err, kErrEos, c);
    if (!ok_region) raise_error(a.err, kErrRegion, c);
    if (!finite) raise_error(a.err, kErrNonFinite, c);
    if (a.irk == 0) {
#pragma unroll
      for (int iv = 0; iv < kNeqMax; ++iv)
        if (iv < neq) a.R[iv * n + c] = rhs[iv];
    } else {
      const double dt = *a.dt;
      const double Vol = m.vol[c];
      double snew[kNeqMax];
#pragma unroll
      for (int iv = 0; iv < kNeqMax; ++iv) {
        if (iv >= neq) break;
        const double S = a.U[iv * n + c];
        double SN;
        if (a.irk == 1) {
          SN = S;  // RK(0): SN = S
          a.SN[iv * n + c] = S;
        } else {
          SN = a.SN[iv * n + c];
        }
        snew[iv] = rk_update(a.irk, S, SN, rhs[iv], dt, Vol);
        a.S_out[iv * n + c] = snew[iv];
        if (a.R) a.R[iv * n + c] = rhs[iv];
      }
      if (a.lambda) lam = cell_lambda(ph, m, c, snew);
    }
  }
  if (a.lambda) block_max_lambda(lam, a.lambda);
}

// RK(irk), RK.c:3-56 from a stored residual.
__global__ void __launch_bounds__(kBlock) k_rk(int irk, int neq, MeshView m, double *__restrict__ S,
                                               double *__restrict__ SN, const double *__restrict__ R,
                                               const double *__restrict__ dtp, double *lambda, Phys ph) {
  const int64_t c = int64_t(blockIdx.x) * kBlock + threadIdx.x;
  double lam = 0.0;
  if (c < m.n) {
    const int64_t n = m.n;
    const double dt = *dtp;
    const double Vol = m.vol[c];
    double snew[kNeqMax] = {0.0, 0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int e = 0; e < kNeqMax; ++e) {
      if (e >= neq) break;
      const int64_t i = e * n + c;
      if (irk == 0) {
        SN[i] = S[i];
        snew[e] = S[i];
      } else {
        snew[e] = rk_update(irk, S[i], SN[i], R[i], dt, Vol);
        S[i] = snew[e];
      }
    }
    if (lambda) lam = cell_lambda(ph, m, c, snew);
  }
  if (lambda) block_max_lambda(lam, lambda);
}

__global__ void __launch_bounds__(kBlock) k_lambda(Phys ph, MeshView m, const double *__restrict__ U,
                                                   double *lambda) {
  const int64_t c = int64_t(blockIdx.x) * kBlock + threadIdx.x;
  double lam = 0.0;
  if (c < m.n) {
    double q[kNeqMax];
    load_state(U, ph.neq, m.n, c, q);
    lam = cell_lambda(ph, m, c, q);
  }
  block_max_lambda(lam, lambda);
}

unsigned grid_of(int64_t n) { return unsigned((n + kBlock - 1) / kBlock); }

}  // namespace

void launch_faceinterp_fp64(const Phys &ph, const MeshView &m, const double *U, double *SF, cudaStream_t st) {
  k_faceinterp<<<grid_of(m.n), kBlock, 0, st>>>(ph, m, U, SF);
}

void launch_gradcalc_fp64(const Phys &ph, const MeshView &m, const double *U, double *SG,
                          unsigned long long *err, cudaStream_t st) {
  k_gradcalc<<<grid_of(m.n), kBlock, 0, st>>>(ph, m, U, SG, err);
}

void launch_residual_fp64(const Phys &ph, const MeshView &m, const ResidualArgs &a, cudaStream_t st) {
  const bool muscl = ph.ischeme == 2, ns = ph.ns == 1;
  if (muscl && ns)
    k_residual<true, true><<<grid_of(m.n), kBlock, 0, st>>>(ph, m, a);
  else if (muscl)
    k_residual<true, false><<<grid_of(m.n), kBlock, 0, st>>>(ph, m, a);
  else if (ns)
    k_residual<false, true><<<grid_of(m.n), kBlock, 0, st>>>(ph, m, a);
  else
    k_residual<false, false><<<grid_of(m.n), kBlock, 0, st>>>(ph, m, a);
}

void launch_rk_fp64(int irk, const Phys &ph, const MeshView &m, double *S, double *SN, const double *R,
                    const double *dt, double *lambda, cudaStream_t st) {
  k_rk<<<grid_of(m.n), kBlock, 0, st>>>(irk, ph.neq, m, S, SN, R, dt, lambda, ph);
}

void launch_lambda_fp64(const Phys &ph, const MeshView &m, const double *U, double *lambda, cudaStream_t st) {
  k_lambda<<<grid_of(m.n), kBlock, 0, st>>>(ph, m, U, lambda);
}

}  // namespace fv
