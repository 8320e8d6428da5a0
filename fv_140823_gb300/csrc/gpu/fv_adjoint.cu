// fvbuild: -fmad=false
//
// Adjoint (vector-Jacobian product) of the FP64 residual:  g = (dR/dU)^T w.
//
// The residual of cell c is a sum over its faces f and sub-faces s of
//   -A_{f,s} Phi(SF_c[f], SF_k[nf]; frame f)          (residual_faces_AMR.c)
// with Phi the HLLC normal flux (hllc_euler.c / compute_wave_speeds.c /
// star_region_euler.c / flux_adv.c) and SF the minmod face values
// (faceinterp.c / reconctruct_V3.c).  The transpose is taken by hand, in
// three gather passes (one thread per cell, fixed order: deterministic, no
// atomics):
//   1. k_adj_flux   reverse of every flux evaluation the cell makes: the
//                   adjoint of its own face value is summed into gL, the one
//                   of the neighbour's face value is stored per evaluation
//                   (gR for a single neighbour, gRh for a 1:4 sub-face);
//   2. k_adj_gsf    adjoint of each face value SF_c[f] = gL + the neighbour
//                   evaluations that read it;
//   3. k_adj_recon  reverse of the reconstruction: own face values and the
//                   face values of the neighbours whose stencil holds c.
// Forward quantities (states, wave speeds, HLLC region, limiter branch) are
// recomputed with the same expressions as the forward kernels, so branch
// decisions match the forward residual exactly.  Scope: model 1, inviscid,
// first order or MUSCL/minmod, inviscid or viscous (4th pass: reverse of the
// Green-Gauss gradients the viscous flux reads), boundary codes other than
// the walls 3 and 4 (inflow 1, transmissive 2), 1:4 faces, periodic meshes.
#include "fv_adjoint.cuh"

#include <cstdio>

namespace fv {

namespace {

constexpr int kBlock = 128;
constexpr int NV = 5;

template <typename T>
struct St {
  T r, ux, uy, uz, e, eint, p, c;
};

// forward face state, model 1 (facevalues.c / facercnstr.c)
template <typename T>
__device__ __forceinline__ void fwd_state(const Phys &ph, const T q[NV], St<T> &s) {
  s.r = q[0];
  s.ux = q[1] / s.r;
  s.uy = q[2] / s.r;
  s.uz = q[3] / s.r;
  s.e = q[4];
  const T gamma = T(ph.gamma), pinf = T(ph.pinf);
  s.eint = (s.e / s.r) - T(0.5) * (s.ux * s.ux + s.uy * s.uy + s.uz * s.uz);
  s.p = s.r * (gamma - T(1.0)) * s.eint - gamma * pinf;
  s.c = sqrt(gamma * (s.p + pinf) / s.r);
}

// reverse of fwd_state: (rb, uxb, uyb, uzb, eb, pb, cb) -> qb (accumulated)
template <typename T>
__device__ __forceinline__ void rev_state(const Phys &ph, const T q[NV], const St<T> &s, T rb, T uxb,
                                          T uyb, T uzb, T eb, T pb, T cb, T qb[NV]) {
  // c = sqrt(X), X = gamma (p + pinf) / r
  const T gamma = T(ph.gamma), pinf = T(ph.pinf);
  const T X = gamma * (s.p + pinf) / s.r;
  const T Xb = cb / (T(2.0) * s.c);
  pb += Xb * gamma / s.r;
  rb -= Xb * X / s.r;
  // p = r (gamma - 1) eint - gamma pinf
  rb += pb * (gamma - T(1.0)) * s.eint;
  const T eintb = pb * s.r * (gamma - T(1.0));
  // eint = e / r - 0.5 |u|^2
  eb += eintb / s.r;
  rb -= eintb * s.e / (s.r * s.r);
  uxb -= eintb * s.ux;
  uyb -= eintb * s.uy;
  uzb -= eintb * s.uz;
  // u = q / r
  qb[1] += uxb / s.r;
  qb[2] += uyb / s.r;
  qb[3] += uzb / s.r;
  rb -= (uxb * s.ux + uyb * s.uy + uzb * s.uz) / s.r;
  qb[0] += rb;
  qb[4] += eb;
  (void)q;
}

// Reverse of the HLLC normal flux Phi = F(U_K).n + S_K (U*_K - U_K) of face
// frame f: given Phib, accumulate qLb and qRb.
template <typename T>
__device__ void hllc_vjp(const Phys &ph, int f, int bc, const T qL[NV], const T qR[NV],
                         const T Phib[NV], const T velLb[3], const T velRb[3], T qLb[NV],
                         T qRb[NV]) {
  const double *fr = ph.frames + 9 * f;
  const T nx = T(fr[0]), ny = T(fr[1]), nz = T(fr[2]), mx = T(fr[3]), my = T(fr[4]), mz = T(fr[5]),
          lx = T(fr[6]), ly = T(fr[7]), lz = T(fr[8]);
  St<T> L, R;
  fwd_state(ph, qL, L);
  fwd_state(ph, qR, R);
  const T uL = L.ux * nx + L.uy * ny + L.uz * nz;
  const T vL = L.ux * mx + L.uy * my + L.uz * mz;
  const T wL = L.ux * lx + L.uy * ly + L.uz * lz;
  const T uR = R.ux * nx + R.uy * ny + R.uz * nz;
  const T vR = R.ux * mx + R.uy * my + R.uz * mz;
  const T wR = R.ux * lx + R.uy * ly + R.uz * lz;
  const T ruL = L.r * uL, ruR = R.r * uR;
  const T a1 = uL + L.c, a2 = uR + R.c, b1 = uL - L.c, b2 = uR - R.c;
  const bool sr_left = a1 > a2, sl_left = b1 < b2;  // max / min of compute_wave_speeds.c:53-54
  const T SR = sr_left ? a1 : a2;
  const T SL = sl_left ? b1 : b2;
  const T nn = rotate_s11(nx, ny, nz, T(1.0));  // d s11 / d p
  const T s11L = rotate_s11(nx, ny, nz, L.p), s11R = rotate_s11(nx, ny, nz, R.p);
  const T num = (L.r * (uL * uL) + s11L) - (R.r * (uR * uR) + s11R) - (SL * ruL) + (SR * ruR);
  const T den = ruL - ruR - (SL * L.r) + (SR * R.r);
  T SS = num / den;
  const bool ss_const = bc == 3;
  if (ss_const) SS = 0.0;
  const bool r1 = 0.0 <= SL;
  const bool r2 = !r1 && (SL <= 0.0) && (0.0 <= SS);
  const bool r3 = !r1 && !r2 && (SS <= 0.0) && (0.0 <= SR);
  const bool left = r1 || r2, star = r2 || r3;
  const St<T> &K = left ? L : R;
  const T *qK = left ? qL : qR;
  const T uK = left ? uL : uR, vK = left ? vL : vR, wK = left ? wL : wR;
  const T SK = left ? SL : SR;

  // bars of K-side quantities
  T rKb = 0, uxKb = 0, uyKb = 0, uzKb = 0, eKb = 0, pKb = 0, uKb = 0, vKb = 0, wKb = 0, SKb = 0, SSb = 0;
  T qKb[NV] = {0, 0, 0, 0, 0};
  // F(U_K).n: [r uK, r ux uK + p nx, r uy uK + p ny, r uz uK + p nz, uK (e + p)]
  {
    const T run = K.r * uK;
    const T runb = Phib[0] + Phib[1] * K.ux + Phib[2] * K.uy + Phib[3] * K.uz;
    uxKb += Phib[1] * run;
    uyKb += Phib[2] * run;
    uzKb += Phib[3] * run;
    pKb += Phib[1] * nx + Phib[2] * ny + Phib[3] * nz + Phib[4] * uK;
    uKb += Phib[4] * (K.e + K.p);
    eKb += Phib[4] * uK;
    rKb += runb * uK;
    uKb += runb * K.r;
  }
  if (star) {
    const T dK = SK - uK, G = SK - SS;
    const T Cs = K.r * dK / G;
    const T T1 = SS * nx + vK * mx + wK * lx, T2 = SS * ny + vK * my + wK * ly,
                 T3 = SS * nz + vK * mz + wK * lz;
    const T Z = K.p / (K.r * dK);
    const T X = SS - uK, Y = SS + Z;
    const T E = (K.e / K.r) + X * Y;
    const T Us[NV] = {Cs, Cs * T1, Cs * T2, Cs * T3, Cs * E};
    T Usb[NV];
    for (int i = 0; i < NV; ++i) {  // FH = SK (Us - qK)
      SKb += Phib[i] * (Us[i] - qK[i]);
      Usb[i] = SK * Phib[i];
      qKb[i] -= SK * Phib[i];
    }
    T Cb = Usb[0] + Usb[1] * T1 + Usb[2] * T2 + Usb[3] * T3 + Usb[4] * E;
    const T T1b = Cs * Usb[1], T2b = Cs * Usb[2], T3b = Cs * Usb[3];
    SSb += T1b * nx + T2b * ny + T3b * nz;
    vKb += T1b * mx + T2b * my + T3b * mz;
    wKb += T1b * lx + T2b * ly + T3b * lz;
    const T Eb = Cs * Usb[4];
    eKb += Eb / K.r;
    rKb -= Eb * K.e / (K.r * K.r);
    const T Xb = Eb * Y, Yb = Eb * X;
    SSb += Xb + Yb;
    uKb -= Xb;
    const T Zb = Yb;
    pKb += Zb / (K.r * dK);
    rKb -= Zb * Z / K.r;
    T dKb = -Zb * Z / dK;
    // Cs = r dK / G
    rKb += Cb * dK / G;
    dKb += Cb * K.r / G;
    const T Gb = -Cb * Cs / G;
    SKb += Gb;
    SSb -= Gb;
    SKb += dKb;
    uKb -= dKb;
  }
  // map the K-side bars to L / R
  T rLb = 0, uxLb = 0, uyLb = 0, uzLb = 0, eLb = 0, pLb = 0, cLb = 0;
  T rRb = 0, uxRb = 0, uyRb = 0, uzRb = 0, eRb = 0, pRb = 0, cRb = 0;
  T uLb = 0, vLb = 0, wLb = 0, uRb = 0, vRb = 0, wRb = 0, SLb = 0, SRb = 0;
  if (left) {
    rLb += rKb; uxLb += uxKb; uyLb += uyKb; uzLb += uzKb; eLb += eKb; pLb += pKb;
    uLb += uKb; vLb += vKb; wLb += wKb; SLb += SKb;
    for (int i = 0; i < NV; ++i) qLb[i] += qKb[i];
  } else {
    rRb += rKb; uxRb += uxKb; uyRb += uyKb; uzRb += uzKb; eRb += eKb; pRb += pKb;
    uRb += uKb; vRb += vKb; wRb += wKb; SRb += SKb;
    for (int i = 0; i < NV; ++i) qRb[i] += qKb[i];
  }
  // S* = num / den (a constant on a slip face)
  if (!ss_const) {
    const T numb = SSb / den, denb = -SSb * num / (den * den);
    // num = (rL uL^2 + s11L) - (rR uR^2 + s11R) - SL ruL + SR ruR
    rLb += numb * uL * uL;
    uLb += numb * T(2.0) * L.r * uL;
    pLb += numb * nn;
    rRb -= numb * uR * uR;
    uRb -= numb * T(2.0) * R.r * uR;
    pRb -= numb * nn;
    SLb -= numb * ruL;
    SRb += numb * ruR;
    T ruLb = -numb * SL, ruRb = numb * SR;
    // den = ruL - ruR - SL rL + SR rR
    ruLb += denb;
    ruRb -= denb;
    SLb -= denb * L.r;
    rLb -= denb * SL;
    SRb += denb * R.r;
    rRb += denb * SR;
    rLb += ruLb * uL;
    uLb += ruLb * L.r;
    rRb += ruRb * uR;
    uRb += ruRb * R.r;
  }
  // SL = min(uL - cL, uR - cR), SR = max(uL + cL, uR + cR)
  if (sl_left) { uLb += SLb; cLb -= SLb; } else { uRb += SLb; cRb -= SLb; }
  if (sr_left) { uLb += SRb; cLb += SRb; } else { uRb += SRb; cRb += SRb; }
  // frame rotations
  uxLb += uLb * nx + vLb * mx + wLb * lx;
  uyLb += uLb * ny + vLb * my + wLb * ly;
  uzLb += uLb * nz + vLb * mz + wLb * lz;
  uxRb += uRb * nx + vRb * mx + wRb * lx;
  uyRb += uRb * ny + vRb * my + wRb * ly;
  uzRb += uRb * nz + vRb * mz + wRb * lz;
  uxLb += velLb[0];  // viscous flux: face-averaged velocity
  uyLb += velLb[1];
  uzLb += velLb[2];
  uxRb += velRb[0];
  uyRb += velRb[1];
  uzRb += velRb[2];
  rev_state(ph, qL, L, rLb, uxLb, uyLb, uzLb, eLb, pLb, cLb, qLb);
  rev_state(ph, qR, R, rRb, uxRb, uyRb, uzRb, eRb, pRb, cRb, qRb);
}

// Reverse of flux_viscous (flux_viscous.c:57-232, turb = 0) contracted with
// the face normal: given the residual weight Phib (= -A w) of one face
// evaluation, the bars of the face-averaged velocity gradients (gb, order
// ux uy uz vx vy vz wx wy wz) and of the face-averaged velocity (ufb) when
// the energy work term is on.  uf and g9 are the forward face averages.
template <typename T>
__device__ __forceinline__ void visc_vjp(const Phys &ph, const double *fr, const T Phib[NV],
                                         const T uf[3], const T g9[9], T gb[9], T ufb[3]) {
  // R_c += A (FV . n): FV bars are -Phib n
  T FVb[NV][3];
#pragma unroll
  for (int v = 0; v < NV; ++v)
#pragma unroll
    for (int d = 0; d < 3; ++d) FVb[v][d] = -Phib[v] * T(fr[d]);
  const T mu = T(ph.visc) + T(0.0);
  const T ux = g9[0], uy = g9[1], uz = g9[2], vx = g9[3], vy = g9[4], vz = g9[5], wx = g9[6], wy = g9[7],
               wz = g9[8];
  T txxb = FVb[1][0], txyb = FVb[1][1] + FVb[2][0], txzb = FVb[1][2] + FVb[3][0];
  T tyyb = FVb[2][1], tyzb = FVb[2][2] + FVb[3][1], tzzb = FVb[3][2];
  ufb[0] = ufb[1] = ufb[2] = 0.0;
  if (ph.eos == 1) {
    const T D = ux + vy + wz;
    const T txx = mu * (T(2.0) * ux - T(2.0 / 3.0) * D), tyy = mu * (T(2.0) * vy - T(2.0 / 3.0) * D);
    const T tzz = mu * (T(2.0) * wz - T(2.0 / 3.0) * D);
    const T txy = mu * (uy + vx), txz = mu * (uz + wx), tyz = mu * (vz + wy);
    const T *e = FVb[4];
    ufb[0] = e[0] * txx + e[1] * txy + e[2] * txz;
    ufb[1] = e[0] * txy + e[1] * tyy + e[2] * tyz;
    ufb[2] = e[0] * txz + e[1] * tyz + e[2] * tzz;
    txxb += uf[0] * e[0];
    txyb += uf[1] * e[0] + uf[0] * e[1];
    txzb += uf[2] * e[0] + uf[0] * e[2];
    tyyb += uf[1] * e[1];
    tyzb += uf[2] * e[1] + uf[1] * e[2];
    tzzb += uf[2] * e[2];
  }
  const T Db = -T(2.0 / 3.0) * mu * (txxb + tyyb + tzzb);
  gb[0] = T(2.0) * mu * txxb + Db;
  gb[4] = T(2.0) * mu * tyyb + Db;
  gb[8] = T(2.0) * mu * tzzb + Db;
  gb[1] = gb[3] = mu * txyb;
  gb[2] = gb[6] = mu * txzb;
  gb[5] = gb[7] = mu * tyzb;
}

template <typename T>
__device__ __forceinline__ void load9(const double *__restrict__ SG, int64_t n, int64_t c, T g[9]) {
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int d = 0; d < 3; ++d) g[a * 3 + d] = T(SG[((1 + a) * 3 + d) * n + c]);
}

template <typename T, typename A_T>
__device__ __forceinline__ void load5(const A_T *__restrict__ A, int64_t n, int64_t c, T q[NV]) {
#pragma unroll
  for (int v = 0; v < NV; ++v) q[v] = T(A[v * n + c]);
}

// value across face f of cell x (deltavalues.c), as the forward computes it
template <typename T>
__device__ __forceinline__ void across(const Phys &ph, const MeshView &m, const double *__restrict__ U, int64_t x,
                                       int f, const T own[NV], T nb[NV]) {
  const int64_t n = m.n;
  const int32_t code = m.nbr[f * n + x];
  if (code >= 0) {
    load5(U, n, code, nb);
  } else if (is_hanging(code)) {
    const int32_t *k = m.hang_nbr + 4 * hang_index(code);
#pragma unroll
    for (int v = 0; v < NV; ++v) nb[v] = 0.0;
    for (int s = 0; s < 4; ++s) {
      const int64_t ks = k[s];
#pragma unroll
      for (int v = 0; v < NV; ++v) nb[v] += T(U[v * n + ks]) / ((T)4);
    }
  } else if (-1 - code == 1) {
#pragma unroll
    for (int v = 0; v < NV; ++v) nb[v] = T(ph.inflow[v]);
  } else {
#pragma unroll
    for (int v = 0; v < NV; ++v) nb[v] = own[v];
  }
}

// Derivatives of the minmod face value SF = q + dcf grad of face g with
// respect to q, the value across g (a) and the value across the opposite face
// (b), per variable (reconctruct_V3.c:17-43).
template <typename T>
__device__ __forceinline__ void recon_deriv(const MeshView &m, int64_t x, int g, const T q[NV],
                                            const T na[NV], const T nb[NV], T dq[NV], T da[NV],
                                            T db[NV]) {
  const int64_t n = m.n;
  const int go = opp_face(g);
  const T dcf = T(m.dcf[g * n + x]), dcc_p = T(m.dcc[g * n + x]), dcc_m = T(m.dcc[go * n + x]);
  const bool bcf = is_boundary(m.nbr[g * n + x]);
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    dq[v] = 1.0;
    da[v] = 0.0;
    db[v] = 0.0;
    if (bcf) continue;
    const T d0 = na[v] - q[v], d1 = nb[v] - q[v];
    if (!(fabs(d0) > T(1e-10))) continue;
    const T product = (-d1 / dcc_m) * (d0 / dcc_p);
    if (!(product > 0.0)) continue;
    if (fabs(-d1 / dcc_m) > fabs(d0 / dcc_p)) {  // grad = d0 / dcc_p
      dq[v] -= dcf / dcc_p;
      da[v] = dcf / dcc_p;
    } else {  // grad = -d1 / dcc_m
      dq[v] += dcf / dcc_m;
      db[v] = -dcf / dcc_m;
    }
  }
}

// 1. reverse of every flux evaluation of cell c
template <typename T>
__device__ __forceinline__ void adj_flux(const Phys &ph, const MeshView &m, const AdjArgsT<T> &a) {
  const int64_t c = int64_t(blockIdx.x) * kBlock + threadIdx.x;
  if (c >= m.n) return;
  const int64_t n = m.n;
  const bool muscl = ph.ischeme == 2;
  const bool ns = ph.ns == 1;
  T w[NV];
  load5(a.w, n, c, w);
  T gown[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // bars of this cell's gradients
  for (int f = 0; f < 6; ++f) {
    const int32_t code = m.nbr[f * n + c];
    const bool boundary = is_boundary(code);
    const int nsub = is_hanging(code) ? 4 : 1;
    T qL[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) qL[v] = muscl ? a.SF[(f * NV + v) * n + c] : a.U[v * n + c];
    T gl[NV] = {0, 0, 0, 0, 0};
    const int nf = m.nbr_face[f * n + c];
    for (int s = 0; s < nsub; ++s) {
      T qR[NV], A;
      int64_t k = -1;
      if (boundary) {
        const int bc = -1 - code;
#pragma unroll
        for (int v = 0; v < NV; ++v) qR[v] = bc == 1 ? T(ph.inflow[v]) : qL[v];
        A = T(m.area[f * n + c]);
      } else {
        if (code >= 0) {
          k = code;
          A = T(m.area[f * n + c]);
        } else {
          const int64_t r = hang_index(code);
          k = m.hang_nbr[4 * r + s];
          A = T(m.hang_area[4 * r + s]);
        }
#pragma unroll
        for (int v = 0; v < NV; ++v) qR[v] = muscl ? a.SF[(nf * NV + v) * n + k] : a.U[v * n + k];
      }
      T Phib[NV], gr[NV] = {0, 0, 0, 0, 0};
#pragma unroll
      for (int v = 0; v < NV; ++v) Phib[v] = -(A)*w[v];
      T vLb[3] = {0, 0, 0}, vRb[3] = {0, 0, 0}, gnb[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      if (ns) {
        // forward face averages: velocities of both face states, gradients of both cells
        T gL9[9], gR9[9], g9[9], uf[3];
        load9(a.SG, n, c, gL9);
        if (k >= 0)
          load9(a.SG, n, k, gR9);
        else
#pragma unroll
          for (int i = 0; i < 9; ++i) gR9[i] = gL9[i];  // a ghost carries the own gradients
#pragma unroll
        for (int i = 0; i < 9; ++i) g9[i] = T(0.5) * (gL9[i] + gR9[i]);
        uf[0] = T(0.5) * (qL[1] / qL[0] + qR[1] / qR[0]);
        uf[1] = T(0.5) * (qL[2] / qL[0] + qR[2] / qR[0]);
        uf[2] = T(0.5) * (qL[3] / qL[0] + qR[3] / qR[0]);
        T gb[9], ufb[3];
        visc_vjp(ph, ph.frames + 9 * f, Phib, uf, g9, gb, ufb);
#pragma unroll
        for (int d = 0; d < 3; ++d) vLb[d] = vRb[d] = T(0.5) * ufb[d];
#pragma unroll
        for (int i = 0; i < 9; ++i) {
          gown[i] += T(0.5) * gb[i];
          gnb[i] = T(0.5) * gb[i];
        }
        if (boundary)
#pragma unroll
          for (int i = 0; i < 9; ++i) gown[i] += gnb[i];
      }
      hllc_vjp(ph, f, boundary ? -1 - code : 0, qL, qR, Phib, vLb, vRb, gl, gr);
      if (boundary) {
        if (-1 - code != 1)  // every supported code but inflow: ghost = own face value
#pragma unroll
          for (int v = 0; v < NV; ++v) gl[v] += gr[v];
      } else if (code >= 0) {
#pragma unroll
        for (int v = 0; v < NV; ++v) a.gR[(f * NV + v) * n + c] = gr[v];
        if (ns)
#pragma unroll
          for (int i = 0; i < 9; ++i) a.gRg[(f * 9 + i) * n + c] = gnb[i];
      } else {
        const int64_t r = hang_index(code);
#pragma unroll
        for (int v = 0; v < NV; ++v) a.gRh[(r * 4 + s) * NV + v] = gr[v];
        if (ns)
#pragma unroll
          for (int i = 0; i < 9; ++i) a.gRgh[(r * 4 + s) * 9 + i] = gnb[i];
      }
    }
#pragma unroll
    for (int v = 0; v < NV; ++v) a.gL[(f * NV + v) * n + c] = gl[v];
  }
  if (ns)
#pragma unroll
    for (int i = 0; i < 9; ++i) a.gG[i * n + c] = gown[i];
}

// 2. adjoint of every face value: own evaluations + neighbour evaluations
template <typename T>
__global__ void __launch_bounds__(kBlock) k_adj_gsf(Phys ph, MeshView m, AdjArgsT<T> a) {
  const int64_t c = int64_t(blockIdx.x) * kBlock + threadIdx.x;
  if (c >= m.n) return;
  const int64_t n = m.n;
  for (int f = 0; f < 6; ++f) {
    const int32_t code = m.nbr[f * n + c];
    T g[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) g[v] = a.gL[(f * NV + v) * n + c];
    if (!is_boundary(code)) {
      const int nf = m.nbr_face[f * n + c];
      if (code >= 0) {
        const int32_t back = m.nbr[nf * n + code];
        if (back >= 0) {  // 1:1 face: the neighbour's single evaluation
#pragma unroll
          for (int v = 0; v < NV; ++v) g[v] += a.gR[(nf * NV + v) * n + code];
        } else {  // the coarse neighbour's 1:4 face: its sub-face that is this cell
          const int64_t r = hang_index(back);
          int sub = 0;
          for (int s = 0; s < 4; ++s)
            if (m.hang_nbr[4 * r + s] == c) sub = s;
#pragma unroll
          for (int v = 0; v < NV; ++v) g[v] += a.gRh[(r * 4 + sub) * NV + v];
        }
      } else {  // this cell's 1:4 face: each fine neighbour's evaluation
        const int32_t *k = m.hang_nbr + 4 * hang_index(code);
        for (int s = 0; s < 4; ++s)
#pragma unroll
          for (int v = 0; v < NV; ++v) g[v] += a.gR[(nf * NV + v) * n + k[s]];
      }
    }
#pragma unroll
    for (int v = 0; v < NV; ++v) a.gSF[(f * NV + v) * n + c] = g[v];
  }
  if (ph.ns != 1) return;
  // adjoint of this cell's gradients: own evaluations + the neighbour
  // evaluations that read them (as s1.g)
  T gt[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) gt[i] = a.gG[i * n + c];
  for (int f = 0; f < 6; ++f) {
    const int32_t code = m.nbr[f * n + c];
    if (is_boundary(code)) continue;
    const int nf = m.nbr_face[f * n + c];
    if (code >= 0) {
      const int32_t back = m.nbr[nf * n + code];
      if (back >= 0) {
#pragma unroll
        for (int i = 0; i < 9; ++i) gt[i] += a.gRg[(nf * 9 + i) * n + code];
      } else {
        const int64_t r = hang_index(back);
        int sub = 0;
        for (int s = 0; s < 4; ++s)
          if (m.hang_nbr[4 * r + s] == c) sub = s;
#pragma unroll
        for (int i = 0; i < 9; ++i) gt[i] += a.gRgh[(r * 4 + sub) * 9 + i];
      }
    } else {
      const int32_t *k = m.hang_nbr + 4 * hang_index(code);
      for (int s = 0; s < 4; ++s)
#pragma unroll
        for (int i = 0; i < 9; ++i) gt[i] += a.gRg[(nf * 9 + i) * n + k[s]];
    }
  }
#pragma unroll
  for (int i = 0; i < 9; ++i) a.gSG[i * n + c] = gt[i];
}

// 3. reverse of the reconstruction
template <typename T>
__device__ __forceinline__ void adj_recon(const Phys &ph, const MeshView &m, const AdjArgsT<T> &a) {
  const int64_t c = int64_t(blockIdx.x) * kBlock + threadIdx.x;
  if (c >= m.n) return;
  const int64_t n = m.n;
  T gu[NV] = {0, 0, 0, 0, 0};
  if (ph.ischeme != 2) {  // first order: every face value is the cell state
    for (int f = 0; f < 6; ++f)
#pragma unroll
      for (int v = 0; v < NV; ++v) gu[v] += a.gSF[(f * NV + v) * n + c];
#pragma unroll
    for (int v = 0; v < NV; ++v) a.out[v * n + c] = gu[v];
    return;
  }
  T q[NV];
  load5(a.U, n, c, q);
  T acr[6][NV];
  for (int f = 0; f < 6; ++f) across(ph, m, a.U, c, f, q, acr[f]);
  // own face values
  for (int g = 0; g < 6; ++g) {
    const int go = opp_face(g);
    T dq[NV], da[NV], db[NV];
    recon_deriv(m, c, g, q, acr[g], acr[go], dq, da, db);
    // across a boundary face whose ghost is the cell's own state (every
    // supported code but inflow) the neighbour value is this cell
    const bool bnd_a = is_boundary(m.nbr[g * n + c]) && -1 - m.nbr[g * n + c] != 1;
    const bool bnd_b = is_boundary(m.nbr[go * n + c]) && -1 - m.nbr[go * n + c] != 1;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const T gs = a.gSF[(g * NV + v) * n + c];
      gu[v] += gs * dq[v];
      if (bnd_a) gu[v] += gs * da[v];  // transmissive ghost across g is this cell
      if (bnd_b) gu[v] += gs * db[v];
    }
  }
  // face values of neighbours whose stencil holds this cell
  for (int f = 0; f < 6; ++f) {
    const int32_t code = m.nbr[f * n + c];
    if (is_boundary(code)) continue;
    const int gk = m.nbr_face[f * n + c];  // the neighbour's face toward this cell
    const int nk = is_hanging(code) ? 4 : 1;
    for (int s = 0; s < nk; ++s) {
      const int64_t k = is_hanging(code) ? int64_t(m.hang_nbr[4 * hang_index(code) + s]) : int64_t(code);
      // this cell counts 1/4 when the neighbour's face is a 1:4 face
      const T wgt = is_hanging(m.nbr[gk * n + k]) ? T(0.25) : T(1.0);
      T qk[NV], ak[NV], bk[NV];
      load5(a.U, n, k, qk);
      across(ph, m, a.U, k, gk, qk, ak);
      across(ph, m, a.U, k, opp_face(gk), qk, bk);
      T dq[NV], da[NV], db[NV];
      // SF_k[gk]: this cell is across gk (the "a" side)
      recon_deriv(m, k, gk, qk, ak, bk, dq, da, db);
#pragma unroll
      for (int v = 0; v < NV; ++v) gu[v] += wgt * a.gSF[(gk * NV + v) * n + k] * da[v];
      // SF_k[opp gk]: this cell is across the opposite face (the "b" side)
      recon_deriv(m, k, opp_face(gk), qk, bk, ak, dq, da, db);
#pragma unroll
      for (int v = 0; v < NV; ++v) gu[v] += wgt * a.gSF[(opp_face(gk) * NV + v) * n + k] * db[v];
    }
  }
#pragma unroll
  for (int v = 0; v < NV; ++v) a.out[v * n + c] = gu[v];
}

// kernels of passes 1 and 3: the FP64 ones with the whole register file
// available, the FP32 ones at four (flux) and six (reconstruction) 128-thread
// blocks per SM, whose register budgets their working sets fit
__global__ void __launch_bounds__(kBlock) k_adj_flux(Phys ph, MeshView m, AdjArgsT<double> a) { adj_flux(ph, m, a); }
__global__ void __launch_bounds__(kBlock) k_adj_recon(Phys ph, MeshView m, AdjArgsT<double> a) {
  adj_recon(ph, m, a);
}
__global__ void __launch_bounds__(kBlock, 4) k_adj_flux_f32(Phys ph, MeshView m, AdjArgsT<float> a) {
  adj_flux(ph, m, a);
}
__global__ void __launch_bounds__(kBlock, 6) k_adj_recon_f32(Phys ph, MeshView m, AdjArgsT<float> a) {
  adj_recon(ph, m, a);
}

// 4. reverse of gradcalc (gradcalc.c:9-47) for the momentum rows the viscous
// flux reads: SG_k[1+a][d] = sum over k's faces 0.5 (q_nb + q_k)[1+a] n_d A / V_k
template <typename T>
__global__ void __launch_bounds__(kBlock) k_adj_grad(Phys ph, MeshView m, AdjArgsT<T> a) {
  const int64_t c = int64_t(blockIdx.x) * kBlock + threadIdx.x;
  if (c >= m.n) return;
  const int64_t n = m.n;
  const T Vc = T(m.vol[c]);
  T coef[3] = {0, 0, 0};  // d SG_c[.][d] / d q_c
  T acc[3] = {0, 0, 0};   // contributions of the neighbours' gradients, per momentum row
  for (int f = 0; f < 6; ++f) {
    const int32_t code = m.nbr[f * n + c];
    const double *fr = ph.frames + 9 * f;
    if (is_boundary(code)) {
      const T own = (-1 - code == 1) ? T(0.5) : T(1.0);  // ghost = own state except at an inflow
      const T A = T(m.area[f * n + c]);
#pragma unroll
      for (int d = 0; d < 3; ++d) coef[d] += own * T(fr[d]) * A / Vc;
      continue;
    }
    const int nf = m.nbr_face[f * n + c];
    const double *fk = ph.frames + 9 * nf;
    const int nsub = is_hanging(code) ? 4 : 1;
    for (int s = 0; s < nsub; ++s) {
      int64_t k;
      T A;  // this cell's (sub-)face area
      if (code >= 0) {
        k = code;
        A = T(m.area[f * n + c]);
      } else {
        const int64_t r = hang_index(code);
        k = m.hang_nbr[4 * r + s];
        A = T(m.hang_area[4 * r + s]);
      }
#pragma unroll
      for (int d = 0; d < 3; ++d) coef[d] += T(0.5) * T(fr[d]) * A / Vc;
      // the area of k's (sub-)face toward this cell
      T Ak;
      const int32_t back = m.nbr[nf * n + k];
      if (back >= 0) {
        Ak = T(m.area[nf * n + k]);
      } else {
        const int64_t r = hang_index(back);
        Ak = T(0.0);
        for (int t = 0; t < 4; ++t)
          if (m.hang_nbr[4 * r + t] == c) Ak = T(m.hang_area[4 * r + t]);
      }
      const T wk = T(0.5) * Ak / T(m.vol[k]);
#pragma unroll
      for (int aa = 0; aa < 3; ++aa)
#pragma unroll
        for (int d = 0; d < 3; ++d) acc[aa] += a.gSG[(aa * 3 + d) * n + k] * T(fk[d]) * wk;
    }
  }
#pragma unroll
  for (int aa = 0; aa < 3; ++aa) {
    T g = acc[aa];
#pragma unroll
    for (int d = 0; d < 3; ++d) g += a.gSG[(aa * 3 + d) * n + c] * coef[d];
    a.out[(1 + aa) * n + c] += g;
  }
}

// Face values of faceinterp.c:21-61 / reconctruct_V3.c:3-57 (minmod,
// iprimtv = 0) in the arithmetic type T, from the FP64 state: the forward
// states the FP32 reverse passes linearise at.  Boundary values as `across`
// forms them (the adjoint's boundary codes: inflow and transmissive).
template <typename T>
__global__ void __launch_bounds__(kBlock) k_adj_faceinterp(Phys ph, MeshView m, const double *__restrict__ U,
                                                           T *__restrict__ SF) {
  const int64_t c = int64_t(blockIdx.x) * kBlock + threadIdx.x;
  if (c >= m.n) return;
  const int64_t n = m.n;
  T q[NV];
  load5(U, n, c, q);
  T acr[6][NV];
  for (int f = 0; f < 6; ++f) across(ph, m, U, c, f, q, acr[f]);
  for (int f = 0; f < 6; ++f) {
    const int fo = opp_face(f);
    const T dcf = T(m.dcf[f * n + c]), dcc_p = T(m.dcc[f * n + c]), dcc_m = T(m.dcc[fo * n + c]);
    const bool bcf = is_boundary(m.nbr[f * n + c]);
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const T d0 = acr[f][v] - q[v], d1 = acr[fo][v] - q[v];
      T grad = T(0.0);
      if (!bcf && fabs(d0) > T(1e-10)) {
        const T sp = d0 / dcc_p, sm = -d1 / dcc_m;
        if (sm * sp > T(0.0)) grad = fabs(sm) > fabs(sp) ? sp : sm;
      }
      SF[(f * NV + v) * n + c] = q[v] + dcf * grad;
    }
  }
}

// w = coef * dt / V * g (the residual weight of a stage's adjoint)
__global__ void k_adj_scale(MeshView m, const double *__restrict__ g, const double *__restrict__ dt, double coef,
                            double *__restrict__ w) {
  const int64_t c = int64_t(blockIdx.x) * kBlock + threadIdx.x;
  if (c >= m.n) return;
  const double s = coef * *dt / m.vol[c];
#pragma unroll
  for (int v = 0; v < NV; ++v) w[v * m.n + c] = s * g[v * m.n + c];
}

// y = alpha * x + beta * y (all variables)
__global__ void k_adj_axpby(int64_t count, double alpha, const double *__restrict__ x, double beta,
                            double *__restrict__ y) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += int64_t(gridDim.x) * blockDim.x)
    y[i] = alpha * x[i] + beta * y[i];
}

unsigned grid_of(int64_t n) { return unsigned((n + kBlock - 1) / kBlock); }

}  // namespace

bool adjoint_supported(const Phys &ph, char *why, size_t whylen) {
  if (ph.model != 1) {
    snprintf(why, whylen, "the adjoint implements model 1 (ideal / stiffened gas)");
    return false;
  }
  return true;
}

void launch_adjoint(const Phys &ph, const MeshView &m, const AdjArgs &a, cudaStream_t st) {
  k_adj_flux<<<grid_of(m.n), kBlock, 0, st>>>(ph, m, a);
  k_adj_gsf<double><<<grid_of(m.n), kBlock, 0, st>>>(ph, m, a);
  k_adj_recon<<<grid_of(m.n), kBlock, 0, st>>>(ph, m, a);
  if (ph.ns == 1) k_adj_grad<double><<<grid_of(m.n), kBlock, 0, st>>>(ph, m, a);
}

void launch_adjoint_f32(const Phys &ph, const MeshView &m, const AdjArgsT<float> &a, cudaStream_t st) {
  k_adj_flux_f32<<<grid_of(m.n), kBlock, 0, st>>>(ph, m, a);
  k_adj_gsf<float><<<grid_of(m.n), kBlock, 0, st>>>(ph, m, a);
  k_adj_recon_f32<<<grid_of(m.n), kBlock, 0, st>>>(ph, m, a);
  if (ph.ns == 1) k_adj_grad<float><<<grid_of(m.n), kBlock, 0, st>>>(ph, m, a);
}

void launch_faceinterp_f32(const Phys &ph, const MeshView &m, const double *U, float *SF, cudaStream_t st) {
  k_adj_faceinterp<float><<<grid_of(m.n), kBlock, 0, st>>>(ph, m, U, SF);
}

void launch_adj_scale(const MeshView &m, const double *g, const double *dt, double coef, double *w, cudaStream_t st) {
  k_adj_scale<<<grid_of(m.n), kBlock, 0, st>>>(m, g, dt, coef, w);
}

void launch_axpby(int64_t count, double alpha, const double *x, double beta, double *y, cudaStream_t st) {
  k_adj_axpby<<<1024, 256, 0, st>>>(count, alpha, x, beta, y);
}

}  // namespace fv
