// Device-side physics of the residual path: face states with their equation
// of state, the HLLC flux, the viscous flux and boundary ghost states.
//
// Each function restates one reference routine and keeps its order of
// operations (C evaluates a+b+c as (a+b)+c; translation units that include
// this header for the FP64 path are compiled with -fmad=false so that no
// product is fused into an add).  Templated on the arithmetic type T: T =
// double is the FP64 path, bit-identical to the reference's C code; T = float
// is the reduced-precision arithmetic of the mixed path.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "fvgpu.h"

namespace fv {

constexpr int kNeqMax = 5;
__host__ __device__ constexpr int opp_face(int f) { return f ^ (f < 4 ? 2 : 1); }  // fcopp: 0<->2 1<->3 4<->5

// Device error codes (error word = code << 40 | cell).
constexpr unsigned long long kErrNonFinite = 1;
constexpr unsigned long long kErrEos = 2;
constexpr unsigned long long kErrRegion = 3;

__device__ __forceinline__ void raise_error(unsigned long long *err, unsigned long long code, int64_t cell) {
  if (err && *((volatile unsigned long long *)err) == 0ull)
    atomicCAS(err, 0ull, (code << 40) | (unsigned long long)(cell & 0xffffffffffll));
}

// Solver constants passed by value to every kernel (lives in the constant
// bank; face frames are indexed by a loop-uniform face index).
struct Phys {
  int model, ns, ischeme, eos, neq, pad;
  double gamma, pinf, visc, ymin;
  double inflow[8];
  double frames[6 * 9];  // per face index: n, t1, t2
};

// Device view of the resident mesh tables.
struct MeshView {
  int64_t n, nhang;
  const int32_t *nbr, *nbr_face;
  const double *area, *dcf, *dcc, *vol;
  const int32_t *hang_nbr;
  const double *hang_area;
};

__device__ __forceinline__ bool is_boundary(int32_t code) { return code < 0 && code > FVGPU_HANG0; }
__device__ __forceinline__ bool is_hanging(int32_t code) { return code <= FVGPU_HANG0; }
__device__ __forceinline__ int64_t hang_index(int32_t code) { return int64_t(FVGPU_HANG0) - code; }

template <typename T>
struct FaceState {
  T r, u, v, w, e, p, c, ymass;
  T vec[kNeqMax];
  T g[9];  // ux uy uz vx vy vz wx wy wz (gradients of rho u, rho v, rho w)
};

// barotropic_eos, barotropic_eos.c:3-30 (pow() is CUDA's: not bit-identical
// to libm, within a few ulp)
template <typename T>
__device__ __forceinline__ void eos_barotropic(FaceState<T> &s) {
  const double nexp = 7.15, beta = 293526643.0, cbar = 1450.0, psat = 2339.0, rsat = 998.2;
  const double r = double(s.r);
  double p = 0.0, c = 0.0;
  if (r >= rsat) {
    p = psat + beta * (pow((r / rsat), nexp) - 1.0);
    c = sqrt(beta * nexp * (pow((r / rsat), (nexp - 1))) / rsat);
  }
  if (r < rsat) {
    p = psat + cbar * ((1.0 / rsat) - (1.0 / r));
    c = sqrt(cbar / (r * r));
  }
  s.p = T(p);
  s.c = T(c);
}

// barotropic_multiphase_eos, barotropic_eos.c:32-129.  Always evaluated in
// FP64: the quadratic pressure inversion is the stiff step.  Returns false
// when neither branch has a real root (the reference exits there).
__device__ __forceinline__ bool eos_mixture(double r, double ymass, double &p_out, double &c_out) {
  const double R_G = 286.0, T_ref = 293.15, r_sat = 998.1618, p_sat = 2340.0;
  const double c_liq = 1482.5, c_mixture = 1.0;
  double c_temp = c_liq;
  double b_coef = c_temp * c_temp * r_sat - p_sat - r * ymass * R_G * T_ref -
                  r * (c_temp * c_temp) * (1.0 - ymass);
  double d_coef = (p_sat - c_temp * c_temp * r_sat) * r * ymass * R_G * T_ref;
  double check = sqrt(b_coef * b_coef - 4.0 * d_coef);
  if (isnan(check)) {
    c_temp = c_mixture;
    b_coef = c_temp * c_temp * r_sat - p_sat - r * ymass * R_G * T_ref -
             r * (c_temp * c_temp) * (1.0 - ymass);
    d_coef = (p_sat - c_temp * c_temp * r_sat) * r * ymass * R_G * T_ref;
    check = sqrt(b_coef * b_coef - 4.0 * d_coef);
    if (isnan(check)) {
      p_out = __longlong_as_double(0x7ff8000000000000ll);
      c_out = c_temp;
      return false;
    }
  }
  const double p1 = (-b_coef + sqrt(b_coef * b_coef - 4.0 * d_coef)) / 2.0;
  const double p2 = (-b_coef - sqrt(b_coef * b_coef - 4.0 * d_coef)) / 2.0;
  p_out = (p1 > p2) ? p1 : p2;
  c_out = c_temp;
  return true;
}

// Face state from conservative values (facercnstr.c:20-59 when clip,
// facevalues.c:113-142 otherwise).  Returns false on an EOS failure.
template <typename T>
__device__ __forceinline__ bool face_state(const Phys &ph, const T *q, bool clip, FaceState<T> &s) {
  bool ok = true;
  s.r = q[0];
  s.u = q[1] / s.r;
  s.v = q[2] / s.r;
  s.w = q[3] / s.r;
  s.vec[0] = s.r;
  s.vec[1] = q[1];
  s.vec[2] = q[2];
  s.vec[3] = q[3];
  if (ph.model == 1) {
    const T gamma = T(ph.gamma), pinf = T(ph.pinf);
    s.e = q[4];
    s.vec[4] = q[4];
    const T e_int = (s.e / s.r) - T(0.5) * (s.u * s.u + s.v * s.v + s.w * s.w);
    s.p = s.r * (gamma - T(1.0)) * e_int - gamma * pinf;
    s.c = sqrt(gamma * (s.p + pinf) / s.r);
  } else if (ph.model == 2) {
    eos_barotropic(s);
  } else {
    s.ymass = q[4] / s.r;
    s.vec[4] = q[4];
    if (clip) {
      const T lo = T(ph.ymin / 1000.0);
      const T hi = T(1.0 - (ph.ymin / 1000.0));
      if (s.ymass < lo) s.ymass = lo;
      if (s.ymass > hi) s.ymass = hi;
    }
    double p, c;
    ok = eos_mixture(double(s.r), double(s.ymass), p, c);
    s.p = T(p);
    s.c = T(c);
  }
  return ok;
}

// Ghost state of a boundary face, bc.c:19-49 (ghost = own state on entry).
template <typename T>
__device__ __forceinline__ void apply_bc(const Phys &ph, int bc, int f, FaceState<T> &g) {
  if (bc == 1) {  // bc_inlet.c -> asinvalues.c:7-44, model 1
    const T rho = T(ph.inflow[0]);
    const T q1 = T(ph.inflow[1]), q2 = T(ph.inflow[2]), q3 = T(ph.inflow[3]), q4 = T(ph.inflow[4]);
    const T gamma = T(ph.gamma), pinf = T(ph.pinf);
    g.r = rho;
    g.u = q1 / rho;
    g.v = q2 / rho;
    g.w = q3 / rho;
    g.vec[0] = rho;
    g.vec[1] = q1;
    g.vec[2] = q2;
    g.vec[3] = q3;
    g.e = q4;
    g.vec[4] = q4;
    const T e_int = (q4 / rho) - T(0.5) * (g.u * g.u + g.v * g.v + g.w * g.w);
    g.p = g.r * (gamma - T(1.0)) * e_int - gamma * pinf;
    g.c = sqrt(gamma * (g.p + pinf) / g.r);
  } else if (bc == 3 || bc == 4) {
    // no reference code (bc_reflective / bc_wall are undefined): slip wall
    // mirrors the normal velocity and momentum, no-slip wall reverses them.
    // The momentum is mirrored as such (not rebuilt as rho * u), so on the
    // axis-aligned faces the tangential components stay exactly the own
    // values and the normal one is exactly negated.
    const T nx = T(ph.frames[9 * f + 0]), ny = T(ph.frames[9 * f + 1]), nz = T(ph.frames[9 * f + 2]);
    if (bc == 3) {
      const T un = (g.u * nx + g.v * ny) + g.w * nz;
      g.u = g.u - T(2.0) * un * nx;
      g.v = g.v - T(2.0) * un * ny;
      g.w = g.w - T(2.0) * un * nz;
      const T mn = (g.vec[1] * nx + g.vec[2] * ny) + g.vec[3] * nz;
      g.vec[1] = g.vec[1] - T(2.0) * mn * nx;
      g.vec[2] = g.vec[2] - T(2.0) * mn * ny;
      g.vec[3] = g.vec[3] - T(2.0) * mn * nz;
    } else {
      g.u = -g.u;
      g.v = -g.v;
      g.w = -g.w;
      g.vec[1] = -g.vec[1];
      g.vec[2] = -g.vec[2];
      g.vec[3] = -g.vec[3];
    }
  }
}

// flux_adv, flux_adv.c:10-45 (st = p I).  The "+ 0" terms are the
// off-diagonal stress entries of the reference; they are kept because they
// turn a -0 product into +0.
template <typename T>
__device__ __forceinline__ void flux_adv(const Phys &ph, const FaceState<T> &s, T F[kNeqMax][3]) {
  F[0][0] = s.u * s.r;
  F[0][1] = s.v * s.r;
  F[0][2] = s.w * s.r;
  F[1][0] = s.r * s.u * s.u + s.p;
  F[1][1] = s.r * s.u * s.v + T(0.0);
  F[1][2] = s.r * s.u * s.w + T(0.0);
  F[2][0] = s.r * s.v * s.u + T(0.0);
  F[2][1] = s.r * s.v * s.v + s.p;
  F[2][2] = s.r * s.v * s.w + T(0.0);
  F[3][0] = s.r * s.w * s.u + T(0.0);
  F[3][1] = s.r * s.w * s.v + T(0.0);
  F[3][2] = s.r * s.w * s.w + s.p;
  if (ph.model == 1) {
    F[4][0] = s.u * (s.e + s.p);
    F[4][1] = s.v * (s.e + s.p);
    F[4][2] = s.w * (s.e + s.p);
  } else if (ph.model == 3) {
    F[4][0] = s.u * s.r * s.ymass;
    F[4][1] = s.v * s.r * s.ymass;
    F[4][2] = s.w * s.r * s.ymass;
  }
}

// (R st R^T)[0][0] for st = p I (rotate_vectors.c:32-90).  The reference
// forms m1[j] = ((0 + R00 st0j) + R01 st1j) + R02 st2j with st's zero
// off-diagonals; for a finite frame each zero product leaves a nonzero
// partial sum unchanged and turns a zero one into +0, so m1[j] == R0j*p + 0
// bit for bit.  The second product is kept as written.
template <typename T>
__device__ __forceinline__ T rotate_s11(T nx, T ny, T nz, T p) {
  const T m0 = nx * p + T(0.0);
  const T m1 = ny * p + T(0.0);
  const T m2 = nz * p + T(0.0);
  return ((T(0.0) + m0 * nx) + m1 * ny) + m2 * nz;
}

// hllc_euler + compute_wave_speeds + star_region_euler:
// hllc_euler.c:3-55, compute_wave_speeds.c:3-88, star_region_euler.c:3-40.
// Writes the normal-flux ingredients F (physical flux tensor) and FH
// (S_K (U*_K - U_K)); returns false if no region matched or S* is NaN.
template <typename T>
__device__ __forceinline__ bool hllc(const Phys &ph, int f, int bc, const FaceState<T> &L,
                                     const FaceState<T> &R, T F[kNeqMax][3], T FH[kNeqMax]) {
  const double *fr = ph.frames + 9 * f;
  const T nx = T(fr[0]), ny = T(fr[1]), nz = T(fr[2]);
  const T mx = T(fr[3]), my = T(fr[4]), mz = T(fr[5]);
  const T lx = T(fr[6]), ly = T(fr[7]), lz = T(fr[8]);
  const T uL = L.u * nx + L.v * ny + L.w * nz;
  const T vL = L.u * mx + L.v * my + L.w * mz;
  const T wL = L.u * lx + L.v * ly + L.w * lz;
  const T uR = R.u * nx + R.v * ny + R.w * nz;
  const T vR = R.u * mx + R.v * my + R.w * mz;
  const T wR = R.u * lx + R.v * ly + R.w * lz;
  const T ruL = L.r * uL;
  const T ruR = R.r * uR;
  const T cL = L.c, cR = R.c;
  const T SR = ((uL + cL) > (uR + cR)) ? (uL + cL) : (uR + cR);
  const T SL = ((uL - cL) < (uR - cR)) ? (uL - cL) : (uR - cR);
  const T s11L = rotate_s11(nx, ny, nz, L.p);
  const T s11R = rotate_s11(nx, ny, nz, R.p);
  T S_S = ((L.r * (uL * uL) + s11L) - (R.r * (uR * uR) + s11R) - (SL * ruL) + (SR * ruR)) /
          (ruL - ruR - (SL * L.r) + (SR * R.r));
  const bool bad_speed = isnan(S_S);
  const int neq = ph.neq;
#pragma unroll
  for (int iv = 0; iv < kNeqMax; ++iv) FH[iv] = T(0.0);
  if (bc == 3) S_S = T(0.0);
  if (T(0.0) <= SL) {
    flux_adv(ph, L, F);
  } else if ((SL <= T(0.0)) && (T(0.0) <= S_S)) {
    flux_adv(ph, L, F);
    const T const_S = L.r * (SL - uL) / (SL - S_S);
    T Us[kNeqMax];
    Us[0] = const_S;
    Us[1] = const_S * (S_S * nx + vL * mx + wL * lx);
    Us[2] = const_S * (S_S * ny + vL * my + wL * ly);
    Us[3] = const_S * (S_S * nz + vL * mz + wL * lz);
    if (ph.model == 1)
      Us[4] = const_S * ((L.e / L.r) + (S_S - uL) * (S_S + (L.p / (L.r * (SL - uL)))));
    else
      Us[4] = const_S * L.ymass;
#pragma unroll
    for (int iv = 0; iv < kNeqMax; ++iv)
      if (iv < neq) FH[iv] = SL * (Us[iv] - L.vec[iv]);
  } else if ((S_S <= T(0.0)) && (T(0.0) <= SR)) {
    flux_adv(ph, R, F);
    const T const_S = R.r * (SR - uR) / (SR - S_S);
    T Us[kNeqMax];
    Us[0] = const_S;
    Us[1] = const_S * (S_S * nx + vR * mx + wR * lx);
    Us[2] = const_S * (S_S * ny + vR * my + wR * ly);
    Us[3] = const_S * (S_S * nz + vR * mz + wR * lz);
    if (ph.model == 1)
      Us[4] = const_S * ((R.e / R.r) + (S_S - uR) * (S_S + (R.p / (R.r * (SR - uR)))));
    else
      Us[4] = const_S * R.ymass;
#pragma unroll
    for (int iv = 0; iv < kNeqMax; ++iv)
      if (iv < neq) FH[iv] = SR * (Us[iv] - R.vec[iv]);
  } else if (SR <= T(0.0)) {
    flux_adv(ph, R, F);
  } else {
    return false;  // "stop if", hllc_euler.c:52-55
  }
  return !bad_speed;
}

// flux_viscous, flux_viscous.c:57-232 with turb = 0.
template <typename T>
__device__ __forceinline__ void flux_viscous(const Phys &ph, const FaceState<T> &s,
                                             const FaceState<T> &s1, T FV[kNeqMax][3]) {
  const T h = T(0.5);
  const T uf = h * (s.u + s1.u), vf = h * (s.v + s1.v), wf = h * (s.w + s1.w);
  const T ux = h * (s.g[0] + s1.g[0]), uy = h * (s.g[1] + s1.g[1]), uz = h * (s.g[2] + s1.g[2]);
  const T vx = h * (s.g[3] + s1.g[3]), vy = h * (s.g[4] + s1.g[4]), vz = h * (s.g[5] + s1.g[5]);
  const T wx = h * (s.g[6] + s1.g[6]), wy = h * (s.g[7] + s1.g[7]), wz = h * (s.g[8] + s1.g[8]);
  const T mu = T(ph.visc) + T(0.0);
  const T two = T(2.0), twothirds = T(2.0 / 3.0);
  const T txx = mu * (two * ux - twothirds * (ux + vy + wz));
  const T tyy = mu * (two * vy - twothirds * (ux + vy + wz));
  const T tzz = mu * (two * wz - twothirds * (ux + vy + wz));
  const T txy = mu * (uy + vx);
  const T txz = mu * (uz + wx);
  const T tyz = mu * (vz + wy);
  FV[0][0] = T(0.0);
  FV[0][1] = T(0.0);
  FV[0][2] = T(0.0);
  FV[1][0] = txx;
  FV[1][1] = txy;
  FV[1][2] = txz;
  FV[2][0] = txy;
  FV[2][1] = tyy;
  FV[2][2] = tyz;
  FV[3][0] = txz;
  FV[3][1] = tyz;
  FV[3][2] = tzz;
  if (ph.eos == 1) {
    FV[4][0] = uf * txx + vf * txy + wf * txz;
    FV[4][1] = uf * txy + vf * tyy + wf * tyz;
    FV[4][2] = uf * txz + vf * tyz + wf * tzz;
  }
}

}  // namespace fv
