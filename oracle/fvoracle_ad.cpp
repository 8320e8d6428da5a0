// fvoracle_ad.cpp -- the oracle's residual and RK step written once over a
// scalar type, for exact directional derivatives.  TEST INFRASTRUCTURE ONLY
// (loaded by tests/ as the checker of libfvgpu's adjoint).
//
// With T = double every expression is evaluated in the same order as
// oracle/fvoracle.c (and so as the reference, residual_faces_AMR.c,
// faceinterp.c, hllc_euler.c, ...); tests check the residual bit for bit.
// With T = Dual (value + one tangent) the same code returns R(U) and the
// Jacobian-vector product J(U) v exactly (forward-mode differentiation of the
// piecewise-smooth residual: branches follow the value part).  The adjoint's
// dot-product test <w, J v> = <J^T w, v> uses these JVPs.
//
// Scope: ideal / stiffened gas (model 1), first order and MUSCL/minmod,
// inviscid or viscous (Green-Gauss gradients, turb = 0, with or without the
// energy work term), boundary codes 1 (inflow) and 2 (transmissive), 1:4
// faces, periodic meshes.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "fvgpu.h"

namespace {

struct Dual {
  double v, d;
  Dual() : v(0.0), d(0.0) {}
  Dual(double x) : v(x), d(0.0) {}
  Dual(double x, double dx) : v(x), d(dx) {}
};
inline Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
inline Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
inline Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
inline Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
inline Dual operator/(Dual a, Dual b) { return Dual(a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)); }
inline Dual &operator+=(Dual &a, Dual b) { return a = a + b; }
inline bool operator<(Dual a, Dual b) { return a.v < b.v; }
inline bool operator>(Dual a, Dual b) { return a.v > b.v; }
inline bool operator<=(Dual a, Dual b) { return a.v <= b.v; }
inline Dual sqrt(Dual a) {
  const double s = std::sqrt(a.v);
  return Dual(s, a.d / (2.0 * s));
}
inline Dual fabs(Dual a) { return a.v < 0.0 ? -a : a; }
inline double val(Dual a) { return a.v; }

// Operation-counting scalar: the FP64 arithmetic of the path, counted per
// kind (sign changes and absolute values are operand modifiers, not counted).
struct OpCounts {
  uint64_t add, mul, div, sqrt;
};
OpCounts g_ops;
struct Cnt {
  double v;
  Cnt() : v(0.0) {}
  Cnt(double x) : v(x) {}
};
inline Cnt operator+(Cnt a, Cnt b) { g_ops.add++; return Cnt(a.v + b.v); }
inline Cnt operator-(Cnt a, Cnt b) { g_ops.add++; return Cnt(a.v - b.v); }
inline Cnt operator-(Cnt a) { return Cnt(-a.v); }
inline Cnt operator*(Cnt a, Cnt b) { g_ops.mul++; return Cnt(a.v * b.v); }
inline Cnt operator/(Cnt a, Cnt b) { g_ops.div++; return Cnt(a.v / b.v); }
inline Cnt &operator+=(Cnt &a, Cnt b) { return a = a + b; }
inline bool operator<(Cnt a, Cnt b) { return a.v < b.v; }
inline bool operator>(Cnt a, Cnt b) { return a.v > b.v; }
inline bool operator<=(Cnt a, Cnt b) { return a.v <= b.v; }
inline Cnt sqrt(Cnt a) { g_ops.sqrt++; return Cnt(std::sqrt(a.v)); }
inline Cnt fabs(Cnt a) { return Cnt(std::fabs(a.v)); }
inline double val(Cnt a) { return a.v; }
inline double val(double a) { return a; }
using std::fabs;
using std::sqrt;

constexpr int NEQ = 5;
const int kOpp[6] = {2, 3, 0, 1, 5, 4};

template <typename T>
struct FState {
  T r, u, v, w, e, p, c;
  T vec[NEQ];
  T g[9];  // ux uy uz vx vy vz wx wy wz: gradients of rho u, rho v, rho w (facercnstr.c:73-85)
};

// facevalues.c:113-129 / facercnstr.c:20-35 (model 1)
template <typename T>
void face_state(const fvgpu_config *cfg, const T *q, FState<T> &s) {
  s.r = q[0];
  s.u = q[1] / s.r;
  s.v = q[2] / s.r;
  s.w = q[3] / s.r;
  for (int k = 0; k < 4; ++k) s.vec[k] = q[k];
  s.e = q[4];
  s.vec[4] = q[4];
  const T e_int = (s.e / s.r) - T(0.5) * (s.u * s.u + s.v * s.v + s.w * s.w);
  s.p = s.r * (T(cfg->gamma) - T(1.0)) * e_int - T(cfg->gamma) * T(cfg->pinf);
  s.c = sqrt(T(cfg->gamma) * (s.p + T(cfg->pinf)) / s.r);
}

// bc_inlet.c -> asinvalues.c:7-44 with the configured inflow state
template <typename T>
void inflow_state(const fvgpu_config *cfg, FState<T> &g) {
  T q[NEQ];
  for (int k = 0; k < NEQ; ++k) q[k] = T(cfg->inflow[k]);
  const T rho = q[0];
  g.r = rho;
  g.u = q[1] / rho;
  g.v = q[2] / rho;
  g.w = q[3] / rho;
  for (int k = 0; k < NEQ; ++k) g.vec[k] = q[k];
  g.e = q[4];
  const T e_int = (q[4] / rho) - T(0.5) * (g.u * g.u + g.v * g.v + g.w * g.w);
  g.p = g.r * (T(cfg->gamma) - T(1.0)) * e_int - T(cfg->gamma) * T(cfg->pinf);
  g.c = sqrt(T(cfg->gamma) * (g.p + T(cfg->pinf)) / g.r);
}

template <typename T>
void flux_adv(const FState<T> &s, T F[NEQ][3]) {
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
  F[4][0] = s.u * (s.e + s.p);
  F[4][1] = s.v * (s.e + s.p);
  F[4][2] = s.w * (s.e + s.p);
}

template <typename T>
T rotate_s11(const double *fr, T p) {
  const T z(0.0);
  T m1[3] = {z, z, z};
  const T st[3][3] = {{p, z, z}, {z, p, z}, {z, z, p}};
  for (int j = 0; j < 3; ++j)
    for (int k = 0; k < 3; ++k) m1[j] += T(fr[k]) * st[k][j];
  T m2 = z;
  for (int k = 0; k < 3; ++k) m2 += m1[k] * T(fr[k]);
  return m2;
}

// hllc_euler.c:3-55 / compute_wave_speeds.c:3-88 / star_region_euler.c:3-40
template <typename T>
void hllc(const double *fr, int bc, const FState<T> &L, const FState<T> &R, T F[NEQ][3], T FH[NEQ]) {
  const T nx(fr[0]), ny(fr[1]), nz(fr[2]), mx(fr[3]), my(fr[4]), mz(fr[5]), lx(fr[6]), ly(fr[7]), lz(fr[8]);
  const T uL = L.u * nx + L.v * ny + L.w * nz;
  const T vL = L.u * mx + L.v * my + L.w * mz;
  const T wL = L.u * lx + L.v * ly + L.w * lz;
  const T uR = R.u * nx + R.v * ny + R.w * nz;
  const T vR = R.u * mx + R.v * my + R.w * mz;
  const T wR = R.u * lx + R.v * ly + R.w * lz;
  const T ruL = L.r * uL, ruR = R.r * uR;
  const T SR = ((uL + L.c) > (uR + R.c)) ? (uL + L.c) : (uR + R.c);
  const T SL = ((uL - L.c) < (uR - R.c)) ? (uL - L.c) : (uR - R.c);
  const T s11L = rotate_s11(fr, L.p), s11R = rotate_s11(fr, R.p);
  T S_S = ((L.r * (uL * uL) + s11L) - (R.r * (uR * uR) + s11R) - (SL * ruL) + (SR * ruR)) /
          (ruL - ruR - (SL * L.r) + (SR * R.r));
  for (int iv = 0; iv < NEQ; ++iv) FH[iv] = T(0.0);
  if (bc == 3) S_S = T(0.0);
  auto star = [&](const FState<T> &s, T SK, T uK, T vK, T wK, T Us[NEQ]) {
    const T const_S = s.r * (SK - uK) / (SK - S_S);
    Us[0] = const_S;
    Us[1] = const_S * (S_S * nx + vK * mx + wK * lx);
    Us[2] = const_S * (S_S * ny + vK * my + wK * ly);
    Us[3] = const_S * (S_S * nz + vK * mz + wK * lz);
    Us[4] = const_S * ((s.e / s.r) + (S_S - uK) * (S_S + (s.p / (s.r * (SK - uK)))));
  };
  T Us[NEQ];
  if (T(0.0) <= SL) {
    flux_adv(L, F);
  } else if ((SL <= T(0.0)) && (T(0.0) <= S_S)) {
    star(L, SL, uL, vL, wL, Us);
    flux_adv(L, F);
    for (int iv = 0; iv < NEQ; ++iv) FH[iv] = SL * (Us[iv] - L.vec[iv]);
  } else if ((S_S <= T(0.0)) && (T(0.0) <= SR)) {
    star(R, SR, uR, vR, wR, Us);
    flux_adv(R, F);
    for (int iv = 0; iv < NEQ; ++iv) FH[iv] = SR * (Us[iv] - R.vec[iv]);
  } else {
    flux_adv(R, F);
  }
}

template <typename T>
struct Mesh {
  const fvgpu_mesh_soa *m;
  int64_t n;
};

// deltavalues.c:3-26 (bc 1: inflow ghost, bc 2: own state)
template <typename T>
void delta_values(const fvgpu_config *cfg, const fvgpu_mesh_soa *m, const T *U, int64_t c, int f, const T *own,
                  T *delta) {
  const int64_t n = m->ncells;
  const int32_t code = m->nbr[int64_t(f) * n + c];
  T nb[NEQ];
  if (code >= 0) {
    for (int v = 0; v < NEQ; ++v) nb[v] = U[int64_t(v) * n + code];
  } else if (code <= FVGPU_HANG0) {
    const int32_t *k = m->hang_nbr + 4 * int64_t(FVGPU_HANG0 - code);
    for (int v = 0; v < NEQ; ++v) nb[v] = T(0.0);
    for (int s = 0; s < 4; ++s)
      for (int v = 0; v < NEQ; ++v) nb[v] += U[int64_t(v) * n + k[s]] / T(double(4));
  } else {
    const int bc = -1 - code;
    if (bc == 1) {
      for (int v = 0; v < NEQ; ++v) nb[v] = T(cfg->inflow[v]);
    } else {
      for (int v = 0; v < NEQ; ++v) nb[v] = own[v];
    }
  }
  for (int v = 0; v < NEQ; ++v) delta[v] = nb[v] - own[v];
}

template <typename T>
void faceinterp(const fvgpu_config *cfg, const fvgpu_mesh_soa *m, const T *U, T *SF) {
  const int64_t n = m->ncells;
  for (int64_t c = 0; c < n; ++c) {
    T own[NEQ];
    for (int v = 0; v < NEQ; ++v) own[v] = U[int64_t(v) * n + c];
    for (int f = 0; f < 6; ++f) {
      const int fo = kOpp[f];
      const double dcf = m->dcf[int64_t(f) * n + c], dcc_p = m->dcc[int64_t(f) * n + c];
      const double dcc_m = m->dcc[int64_t(fo) * n + c];
      T d0[NEQ], d1[NEQ];
      delta_values(cfg, m, U, c, fo, own, d1);
      delta_values(cfg, m, U, c, f, own, d0);
      const int32_t code = m->nbr[int64_t(f) * n + c];
      const bool bcf = code < 0 && code > FVGPU_HANG0;
      for (int iv = 0; iv < NEQ; ++iv) {
        T grad(0.0);
        if (!bcf) {
          if (val(fabs(d0[iv])) > 1e-10) {
            const T product = (-d1[iv] / T(dcc_m)) * (d0[iv] / T(dcc_p));
            if (val(product) > 0.0) {
              if (val(fabs(-d1[iv] / T(dcc_m))) > val(fabs(d0[iv] / T(dcc_p))))
                grad = d0[iv] / T(dcc_p);
              else
                grad = -d1[iv] / T(dcc_m);
            } else {
              grad = T(0.0);
            }
          }
        }
        SF[(int64_t(f) * NEQ + iv) * n + c] = own[iv] + T(dcf) * grad;
      }
    }
  }
}

// gradcalc.c:9-47 (Green-Gauss, first-order face states; oracle fvo_gradcalc)
template <typename T>
void gradcalc(const fvgpu_config *cfg, const fvgpu_mesh_soa *m, const T *U, T *SG) {
  const int64_t n = m->ncells;
  for (int64_t c = 0; c < n; ++c) {
    T g[NEQ + 1][3];
    for (int iv = 0; iv <= NEQ; ++iv) g[iv][0] = g[iv][1] = g[iv][2] = T(0.0);
    T own[NEQ];
    for (int v = 0; v < NEQ; ++v) own[v] = U[int64_t(v) * n + c];
    const double Vol = m->vol[c];
    for (int f = 0; f < 6; ++f) {
      const int32_t code = m->nbr[int64_t(f) * n + c];
      const double *fr = m->frames + 9 * f;
      const int nsub = code <= FVGPU_HANG0 ? 4 : 1;
      for (int ing = 0; ing < nsub; ++ing) {
        FState<T> s, s1;
        face_state(cfg, own, s);
        double A;
        if (code >= 0) {
          T q[NEQ];
          for (int v = 0; v < NEQ; ++v) q[v] = U[int64_t(v) * n + code];
          face_state(cfg, q, s1);
          A = m->area[int64_t(f) * n + c];
        } else if (code <= FVGPU_HANG0) {
          const int64_t r = FVGPU_HANG0 - code;
          T q[NEQ];
          for (int v = 0; v < NEQ; ++v) q[v] = U[int64_t(v) * n + m->hang_nbr[4 * r + ing]];
          face_state(cfg, q, s1);
          A = m->hang_area[4 * r + ing];
        } else {
          face_state(cfg, own, s1);
          if (-1 - code == 1) inflow_state(cfg, s1);
          A = m->area[int64_t(f) * n + c];
        }
        for (int iv = 0; iv < NEQ; ++iv)
          for (int d = 0; d < 3; ++d) g[iv][d] += T(0.5) * (s1.vec[iv] + s.vec[iv]) * T(fr[d]) * T(A) / T(Vol);
        for (int d = 0; d < 3; ++d) g[NEQ][d] += T(0.5) * (s1.p + s.p) * T(fr[d]) * T(A) / T(Vol);
      }
    }
    for (int iv = 0; iv <= NEQ; ++iv)
      for (int d = 0; d < 3; ++d) SG[(int64_t(iv) * 3 + d) * n + c] = g[iv][d];
  }
}

// flux_viscous.c:57-232 with turb = 0 (oracle flux_visc)
template <typename T>
void flux_visc(const fvgpu_config *cfg, const FState<T> &s, const FState<T> &s1, T FV[NEQ][3]) {
  const T h(0.5);
  const T uf = h * (s.u + s1.u), vf = h * (s.v + s1.v), wf = h * (s.w + s1.w);
  const T ux = h * (s.g[0] + s1.g[0]), uy = h * (s.g[1] + s1.g[1]), uz = h * (s.g[2] + s1.g[2]);
  const T vx = h * (s.g[3] + s1.g[3]), vy = h * (s.g[4] + s1.g[4]), vz = h * (s.g[5] + s1.g[5]);
  const T wx = h * (s.g[6] + s1.g[6]), wy = h * (s.g[7] + s1.g[7]), wz = h * (s.g[8] + s1.g[8]);
  const T mu = T(cfg->visc) + T(0.0);
  const T txx = mu * (T(2.0) * ux - T(2.0 / 3.0) * (ux + vy + wz));
  const T tyy = mu * (T(2.0) * vy - T(2.0 / 3.0) * (ux + vy + wz));
  const T tzz = mu * (T(2.0) * wz - T(2.0 / 3.0) * (ux + vy + wz));
  const T txy = mu * (uy + vx);
  const T txz = mu * (uz + wx);
  const T tyz = mu * (vz + wy);
  FV[0][0] = FV[0][1] = FV[0][2] = T(0.0);
  FV[1][0] = txx;
  FV[1][1] = txy;
  FV[1][2] = txz;
  FV[2][0] = txy;
  FV[2][1] = tyy;
  FV[2][2] = tyz;
  FV[3][0] = txz;
  FV[3][1] = tyz;
  FV[3][2] = tzz;
  if (cfg->eos == 1) {
    FV[4][0] = uf * txx + vf * txy + wf * txz;
    FV[4][1] = uf * txy + vf * tyy + wf * tyz;
    FV[4][2] = uf * txz + vf * tyz + wf * tzz;
  }
}

template <typename T>
void rhs(const fvgpu_config *cfg, const fvgpu_mesh_soa *m, const T *U, const T *SF, const T *SG, T *R) {
  const int64_t n = m->ncells;
  const bool muscl = cfg->ischeme == 2;
  const bool ns = cfg->ns == 1;
  auto grad9 = [&](int64_t k, T *g) {
    for (int a = 0; a < 3; ++a)
      for (int d = 0; d < 3; ++d) g[a * 3 + d] = SG[(int64_t(1 + a) * 3 + d) * n + k];
  };
  for (int64_t c = 0; c < n; ++c) {
    T acc[NEQ];
    for (int iv = 0; iv < NEQ; ++iv) acc[iv] = T(0.0);
    T FV[NEQ][3];
    for (int iv = 0; iv < NEQ; ++iv) FV[iv][0] = FV[iv][1] = FV[iv][2] = T(0.0);
    for (int f = 0; f < 6; ++f) {
      const int32_t code = m->nbr[int64_t(f) * n + c];
      const double *fr = m->frames + 9 * f;
      const bool boundary = code < 0 && code > FVGPU_HANG0;
      const int nsub = code <= FVGPU_HANG0 ? 4 : 1;
      T flux_face[NEQ];
      for (int iv = 0; iv < NEQ; ++iv) flux_face[iv] = T(0.0);
      T qown[NEQ];
      for (int v = 0; v < NEQ; ++v) qown[v] = muscl ? SF[(int64_t(f) * NEQ + v) * n + c] : U[int64_t(v) * n + c];
      FState<T> s;
      face_state(cfg, qown, s);
      if (ns) grad9(c, s.g);
      for (int ineig = 0; ineig < nsub; ++ineig) {
        FState<T> s1;
        double A;
        if (boundary) {
          s1 = s;
          if (-1 - code == 1) inflow_state(cfg, s1);
          A = m->area[int64_t(f) * n + c];
        } else {
          int64_t k;
          if (code >= 0) {
            k = code;
            A = m->area[int64_t(f) * n + c];
          } else {
            const int64_t r = FVGPU_HANG0 - code;
            k = m->hang_nbr[4 * r + ineig];
            A = m->hang_area[4 * r + ineig];
          }
          const int nf = m->nbr_face[int64_t(f) * n + c];
          T q[NEQ];
          for (int v = 0; v < NEQ; ++v) q[v] = muscl ? SF[(int64_t(nf) * NEQ + v) * n + k] : U[int64_t(v) * n + k];
          face_state(cfg, q, s1);
          if (ns) grad9(k, s1.g);
        }
        if (ns) flux_visc(cfg, s, s1, FV);
        T F[NEQ][3], FH[NEQ];
        hllc(fr, boundary ? -1 - code : 0, s, s1, F, FH);
        for (int iv = 0; iv < NEQ; ++iv)
          flux_face[iv] += -T(A) * (((F[iv][0] - FV[iv][0]) * T(fr[0]) + (F[iv][1] - FV[iv][1]) * T(fr[1]) +
                                     (F[iv][2] - FV[iv][2]) * T(fr[2])) +
                                    FH[iv]);
      }
      for (int iv = 0; iv < NEQ; ++iv) acc[iv] += flux_face[iv];
    }
    for (int iv = 0; iv < NEQ; ++iv) R[int64_t(iv) * n + c] = acc[iv];
  }
}

template <typename T>
void residual(const fvgpu_config *cfg, const fvgpu_mesh_soa *m, const T *U, T *R) {
  std::vector<T> SF, SG;
  if (cfg->ischeme == 2) {
    SF.resize(size_t(6 * NEQ * m->ncells));
    faceinterp(cfg, m, U, SF.data());
  }
  if (cfg->ns == 1) {
    SG.resize(size_t(3 * (NEQ + 1) * m->ncells));
    gradcalc(cfg, m, U, SG.data());
  }
  rhs(cfg, m, U, cfg->ischeme == 2 ? SF.data() : nullptr, cfg->ns == 1 ? SG.data() : nullptr, R);
}

// RK.c:16-47 stage formulas
template <typename T>
void rk(int irk, double dt, const fvgpu_mesh_soa *m, T *S, T *SN, const T *R) {
  const int64_t n = m->ncells;
  for (int64_t c = 0; c < n; ++c) {
    const double Vol = m->vol[c];
    for (int e = 0; e < NEQ; ++e) {
      const int64_t i = int64_t(e) * n + c;
      switch (irk) {
        case 0: SN[i] = S[i]; break;
        case 1: S[i] = SN[i] + T(dt) * (T(1.0) / T(Vol)) * R[i]; break;
        case 2: S[i] = T(3.0 / 4.0) * SN[i] + T(1.0 / 4.0) * S[i] + T(1.0 / 4.0) * T(dt) * R[i] / T(Vol); break;
        case 3: S[i] = T(1.0 / 3.0) * SN[i] + T(2.0 / 3.0) * S[i] + T(2.0 / 3.0) * T(dt) * R[i] / T(Vol); break;
        case 4: S[i] = T(1.0 / 2.0) * SN[i] + T(1.0 / 2.0) * S[i] + T(1.0 / 2.0) * T(dt) * R[i] / T(Vol); break;
        default: break;
      }
    }
  }
}

}  // namespace

extern "C" {

// R(U) with T = double (bit-identical to fvo_rhs after fvo_faceinterp).
int fvo_ad_residual(const fvgpu_config *cfg, const fvgpu_mesh_soa *m, const double *U, double *R) {
  if (cfg->model != 1) return -1;
  residual<double>(cfg, m, U, R);
  return 0;
}

// R(U) and J(U) V in one forward-mode pass.
int fvo_ad_jvp(const fvgpu_config *cfg, const fvgpu_mesh_soa *m, const double *U, const double *V, double *R,
               double *JV) {
  if (cfg->model != 1) return -1;
  const int64_t N = NEQ * m->ncells;
  std::vector<Dual> Ud(static_cast<size_t>(N)), Rd(static_cast<size_t>(N));
  for (int64_t i = 0; i < N; ++i) Ud[size_t(i)] = Dual(U[i], V[i]);
  residual<Dual>(cfg, m, Ud.data(), Rd.data());
  for (int64_t i = 0; i < N; ++i) {
    if (R) R[i] = Rd[size_t(i)].v;
    JV[i] = Rd[size_t(i)].d;
  }
  return 0;
}

// nsteps RK steps at fixed dt from U with tangent V: final state and its
// tangent (the directional derivative of the step map).
int fvo_ad_steps_jvp(const fvgpu_config *cfg, const fvgpu_mesh_soa *m, const int *stages, int nstages, double dt,
                     int nsteps, const double *U, const double *V, double *S_out, double *JV) {
  if (cfg->model != 1) return -1;
  const int64_t N = NEQ * m->ncells;
  std::vector<Dual> S(static_cast<size_t>(N)), SN(static_cast<size_t>(N)), R(static_cast<size_t>(N));
  for (int64_t i = 0; i < N; ++i) S[size_t(i)] = Dual(U[i], V[i]);
  for (int step = 0; step < nsteps; ++step) {
    rk<Dual>(0, dt, m, S.data(), SN.data(), R.data());
    for (int k = 0; k < nstages; ++k) {
      residual<Dual>(cfg, m, S.data(), R.data());
      rk<Dual>(stages[k], dt, m, S.data(), SN.data(), R.data());
    }
  }
  for (int64_t i = 0; i < N; ++i) {
    if (S_out) S_out[i] = S[size_t(i)].v;
    JV[i] = S[size_t(i)].d;
  }
  return 0;
}

// FP64 operations of nsteps RK steps from U (the FP64 path's arithmetic,
// counted once per operation of the restated expressions): counts[0..3] =
// additions / subtractions, multiplications, divisions, square roots.
int fvo_ad_count_steps(const fvgpu_config *cfg, const fvgpu_mesh_soa *m, const int *stages, int nstages, double dt,
                       int nsteps, const double *U, uint64_t *counts) {
  if (cfg->model != 1) return -1;
  const int64_t N = NEQ * m->ncells;
  std::vector<Cnt> S(static_cast<size_t>(N)), SN(static_cast<size_t>(N)), R(static_cast<size_t>(N));
  for (int64_t i = 0; i < N; ++i) S[size_t(i)] = Cnt(U[i]);
  g_ops = OpCounts{0, 0, 0, 0};
  for (int step = 0; step < nsteps; ++step) {
    rk<Cnt>(0, dt, m, S.data(), SN.data(), R.data());
    for (int k = 0; k < nstages; ++k) {
      residual<Cnt>(cfg, m, S.data(), R.data());
      rk<Cnt>(stages[k], dt, m, S.data(), SN.data(), R.data());
    }
  }
  counts[0] = g_ops.add;
  counts[1] = g_ops.mul;
  counts[2] = g_ops.div;
  counts[3] = g_ops.sqrt;
  return 0;
}

// FP64 operations of one stage split by kernel: counts[0..3] faceinterp,
// counts[4..7] residual with the fused RK(irk) update (kinds as above).
int fvo_ad_count_stage(const fvgpu_config *cfg, const fvgpu_mesh_soa *m, int irk, double dt, const double *U,
                       uint64_t *counts) {
  if (cfg->model != 1) return -1;
  const int64_t N = NEQ * m->ncells;
  std::vector<Cnt> S(static_cast<size_t>(N)), SN(static_cast<size_t>(N)), R(static_cast<size_t>(N));
  std::vector<Cnt> SF(static_cast<size_t>(6 * N));
  for (int64_t i = 0; i < N; ++i) S[size_t(i)] = SN[size_t(i)] = Cnt(U[i]);
  g_ops = OpCounts{0, 0, 0, 0};
  if (cfg->ischeme == 2) faceinterp(cfg, m, S.data(), SF.data());
  counts[0] = g_ops.add;
  counts[1] = g_ops.mul;
  counts[2] = g_ops.div;
  counts[3] = g_ops.sqrt;
  g_ops = OpCounts{0, 0, 0, 0};
  std::vector<Cnt> SG(static_cast<size_t>(3 * (NEQ + 1) * m->ncells));
  if (cfg->ns == 1) gradcalc(cfg, m, S.data(), SG.data());
  rhs(cfg, m, S.data(), cfg->ischeme == 2 ? SF.data() : nullptr, SG.data(), R.data());
  rk<Cnt>(irk, dt, m, S.data(), SN.data(), R.data());
  counts[4] = g_ops.add;
  counts[5] = g_ops.mul;
  counts[6] = g_ops.div;
  counts[7] = g_ops.sqrt;
  return 0;
}

}  // extern "C"
