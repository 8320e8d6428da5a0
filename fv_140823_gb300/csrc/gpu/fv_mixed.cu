// fvbuild: -fmad=false
//
// FP32-mixed path: one fused kernel per RK stage.
//
// Arithmetic.  Reconstruction, equation of state and HLLC fluxes run in FP32
// (the mixture EOS pressure inversion stays FP64).  The state is kept in FP64
// as the step-start state SN; a stage k carries only the FP32 increment
// D_k = S_k - SN, so the RK stage formulas of RK.c become
//     RK(1): D1 = dt/V R(S0)                      S1 = SN + D1
//     RK(2): D2 = 1/4 (D1 + dt/V R(S1))           S2 = 3/4 SN + 1/4 S1 + 1/4 dt/V R
//     RK(3): D3 = 2/3 (D2 + dt/V R(S2))           S3 = 1/3 SN + 2/3 S2 + 2/3 dt/V R
//     RK(4): D  = 1/2 (D1 + dt/V R(S1))           (SSP-RK2 second stage)
// and the step ends with one FP64 add per variable, SN <- SN + D_last.  The
// per-stage increments are small against the state, so their FP32 rounding
// is ~1e-8 of the state per stage while every add into the state itself is
// FP64.  On GB300 the FP64 pipe runs at ~1/70 of FP32; this keeps the FP64
// work to a few operations per cell and step, which is what lets the stage
// kernel run at the HBM limit.
//
// Work decomposition.  One thread per cell, blocks of kBlock consecutive cells
// (Morton order: an 8x8x4 brick of a uniform octree).  Phases:
//   A  stage state S = SN + D of the block's cells into shared memory
//   B  MUSCL/minmod face values of the thread's own 6 faces (faceinterp.c /
//      reconctruct_V3.c) into shared memory
//   C  flux of each face computed once, canonically from the face's lower
//      cell (the one whose +x/+y/+z face it is): threads compute their own
//      + faces and publish them in shared memory; the upper cell reads it, or
//      recomputes the same canonical flux bit for bit when the lower cell is
//      in another block or the face is a 1:4 sub-face.  Equal and opposite
//      contributions -> exactly conservative and deterministic.
//   D  residual, RK stage update, (last stage) FP64 state and CFL radius.
// Geometry comes from per-level tables (octree-regular meshes): a packed
// per-cell code (level + face relations) replaces the FP64 face tables.
#include <cstdio>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "fv_mixed.cuh"

namespace fv {

namespace {

constexpr int kBlock = 256;
constexpr int kMaxLevel = 18;
constexpr int kRelSame = 0, kRelFiner = 1, kRelCoarser = 2, kRelBoundary = 3;
// per (level, face, relation): dcf, 1/dcc, area, pad
constexpr int kGeoStride = 4;
constexpr int kGeoEntries = (kMaxLevel + 1) * 6 * 4;

struct GeoTables {
  float face[kGeoEntries * kGeoStride];
  float sub_area[(kMaxLevel + 1) * 6];
  float vol[kMaxLevel + 1];
  float inv_vol[kMaxLevel + 1];
  float inv2vol[kMaxLevel + 1];  // 1 / (2 V): CFL radius
};

__host__ __device__ constexpr int geo_index(int level, int f, int rel) { return ((level * 6 + f) * 4 + rel); }

// + faces: normals +x (1), +y (2), +z (5); their slot in the flux table
__host__ __device__ constexpr bool is_plus_face(int f) { return f == 1 || f == 2 || f == 5; }
__device__ __forceinline__ int plus_slot(int f) { return f == 1 ? 0 : (f == 2 ? 1 : 2); }

// FP32 constants of the mixed path, converted once on the host (FP64 -> FP32
// conversions inside the kernel would run on GB300's slow FP64 pipe).
struct MixedConst {
  float fr[54];      // face frames n, t1, t2 per face index
  float gamma, pinf, gm1, gpinf;
  float ylo, yhi;    // mass-fraction clip (facercnstr.c:43-44)
  float inflow[kNeqMax];
  int model, neq, ischeme, pad;
};

struct StageArgs {
  int64_t n;
  const int32_t *nbr;       // [6][n]
  const int32_t *geom;      // [n]: level | rel_f << (5 + 2 f)
  const int32_t *hang_nbr;  // [nhang][4]
  const GeoTables *geo;
  const double *SN;         // [neq][n] step-start state
  const float *Din;         // [neq][n] stage-input increment (null: zero)
  float *Dout;              // [neq][n]
  double *SNout;            // [neq][n] last stage: SN + D
  const double *dt;
  double *lambda;           // last stage: CFL radius of the new state
  int irk;
  int last;
  unsigned long long *err;
};

__device__ __forceinline__ int level_of(int32_t g) { return g & 31; }
__device__ __forceinline__ int rel_of(int32_t g, int f) { return (g >> (5 + 2 * f)) & 3; }

__device__ __forceinline__ const float *geo_face(const GeoTables *G, int level, int f, int rel) {
  return G->face + geo_index(level, f, rel) * kGeoStride;
}

// FP32 face state (facercnstr.c / facevalues.c with fast reciprocals).
struct FS {
  float r, u, v, w, e, p, c, y;
  float q[kNeqMax];
};

__device__ __forceinline__ bool mixed_face_state(const MixedConst &mc, const float *q, bool clip, FS &s) {
  s.r = q[0];
  const float rinv = __frcp_rn(s.r);
  s.u = q[1] * rinv;
  s.v = q[2] * rinv;
  s.w = q[3] * rinv;
#pragma unroll
  for (int v = 0; v < kNeqMax; ++v) s.q[v] = q[v];
  if (mc.model == 1) {
    s.e = q[4];
    const float ke = fmaf(s.w, s.w, fmaf(s.v, s.v, s.u * s.u));
    const float e_int = fmaf(-0.5f, ke, s.e * rinv);
    s.p = fmaf(s.r * mc.gm1, e_int, -mc.gpinf);
    s.c = __fsqrt_rn(mc.gamma * (s.p + mc.pinf) * rinv);
    s.y = 0.0f;
    return true;
  }
  // model 3: mass fraction in FP32, pressure inversion in FP64
  s.y = q[4] * rinv;
  if (clip) {
    s.y = s.y < mc.ylo ? mc.ylo : s.y;
    s.y = s.y > mc.yhi ? mc.yhi : s.y;
  }
  double p, c;
  const bool ok = eos_mixture(double(s.r), double(s.y), p, c);
  s.p = float(p);
  s.c = float(c);
  s.e = 0.0f;
  return ok;
}

// Normal flux through a face with unit normal n (frame f): HLLC of
// hllc_euler.c / compute_wave_speeds.c / star_region_euler.c, contracted
// with n as residual_faces_AMR.c:145-149 does (F.n + F_HLLC).
__device__ __forceinline__ bool mixed_hllc_normal(const MixedConst &mc, int f, int bc, const FS &L, const FS &R,
                                                  float out[kNeqMax]) {
  const float *fr = mc.fr + 9 * f;
  const float nx = fr[0], ny = fr[1], nz = fr[2];
  const float mx = fr[3], my = fr[4], mz = fr[5];
  const float lx = fr[6], ly = fr[7], lz = fr[8];
  const float uL = fmaf(L.w, nz, fmaf(L.v, ny, L.u * nx));
  const float vL = fmaf(L.w, mz, fmaf(L.v, my, L.u * mx));
  const float wL = fmaf(L.w, lz, fmaf(L.v, ly, L.u * lx));
  const float uR = fmaf(R.w, nz, fmaf(R.v, ny, R.u * nx));
  const float vR = fmaf(R.w, mz, fmaf(R.v, my, R.u * mx));
  const float wR = fmaf(R.w, lz, fmaf(R.v, ly, R.u * lx));
  const float SR = fmaxf(uL + L.c, uR + R.c);
  const float SL = fminf(uL - L.c, uR - R.c);
  const float ruL = L.r * uL, ruR = R.r * uR;
  const float nn = (nx * nx + ny * ny) + nz * nz;  // (R st R^T)[0][0] = p |n|^2
  const float num = fmaf(SR, ruR, fmaf(-SL, ruL, fmaf(ruL, uL, L.p * nn) - fmaf(ruR, uR, R.p * nn)));
  const float den = fmaf(SR, R.r, fmaf(-SL, L.r, ruL - ruR));
  float S_S = __fdividef(num, den);
  const bool ok = !isnan(S_S);
  if (bc == 3) S_S = 0.0f;
  // region selection in the order of hllc_euler.c:18-50
  const bool r1 = 0.0f <= SL;
  const bool r2 = !r1 && (SL <= 0.0f) && (0.0f <= S_S);
  const bool r3 = !r1 && !r2 && (S_S <= 0.0f) && (0.0f <= SR);
  const bool r4 = !r1 && !r2 && !r3 && (SR <= 0.0f);
  const bool left = r1 || r2;
  const bool star = r2 || r3;
  const FS &K = left ? L : R;
  const float uK = left ? uL : uR, vK = left ? vL : vR, wK = left ? wL : wR;
  const float SK = left ? SL : SR;
  // physical flux F(U_K) . n
  const float un = uK;  // u_K . n
  float Fn[kNeqMax];
  Fn[0] = K.r * un;
  Fn[1] = fmaf(K.p, nx, K.r * K.u * un);
  Fn[2] = fmaf(K.p, ny, K.r * K.v * un);
  Fn[3] = fmaf(K.p, nz, K.r * K.w * un);
  if (mc.model == 1)
    Fn[4] = (K.e + K.p) * un;
  else
    Fn[4] = K.r * K.y * un;
  if (star) {
    const float dK = SK - uK;
    const float cS = __fdividef(K.r * dK, SK - S_S);
    const float us0 = cS * fmaf(wK, lx, fmaf(vK, mx, S_S * nx));
    const float us1 = cS * fmaf(wK, ly, fmaf(vK, my, S_S * ny));
    const float us2 = cS * fmaf(wK, lz, fmaf(vK, mz, S_S * nz));
    float us4;
    if (mc.model == 1)
      us4 = cS * fmaf(S_S - uK, S_S + __fdividef(K.p, K.r * dK), K.e * __frcp_rn(K.r));
    else
      us4 = cS * K.y;
    Fn[0] = fmaf(SK, cS - K.q[0], Fn[0]);
    Fn[1] = fmaf(SK, us0 - K.q[1], Fn[1]);
    Fn[2] = fmaf(SK, us1 - K.q[2], Fn[2]);
    Fn[3] = fmaf(SK, us2 - K.q[3], Fn[3]);
    Fn[4] = fmaf(SK, us4 - K.q[4], Fn[4]);
  }
  const bool region = r1 || r2 || r3 || r4;
#pragma unroll
  for (int v = 0; v < kNeqMax; ++v) out[v] = Fn[v];
  return ok && region;
}

// Boundary ghost (bc.c) from the own face state.
__device__ __forceinline__ void mixed_ghost(const MixedConst &mc, int bc, int f, FS &g) {
  if (bc == 1) {
    mixed_face_state(mc, mc.inflow, false, g);
  } else if (bc == 3 || bc == 4) {
    const float nx = mc.fr[9 * f], ny = mc.fr[9 * f + 1], nz = mc.fr[9 * f + 2];
    if (bc == 3) {
      const float un = g.u * nx + g.v * ny + g.w * nz;
      g.u -= 2.0f * un * nx;
      g.v -= 2.0f * un * ny;
      g.w -= 2.0f * un * nz;
    } else {
      g.u = -g.u;
      g.v = -g.v;
      g.w = -g.w;
    }
    g.q[1] = g.r * g.u;
    g.q[2] = g.r * g.v;
    g.q[3] = g.r * g.w;
  }
}

struct Ctx {
  const StageArgs &a;
  const MixedConst &ph;
  int64_t c0;
  const float (*st)[kBlock];  // [neq][kBlock] block states
  __device__ Ctx(const StageArgs &a_, const MixedConst &ph_, int64_t c0_, const float (*st_)[kBlock])
      : a(a_), ph(ph_), c0(c0_), st(st_) {}
  __device__ __forceinline__ bool in_block(int64_t x) const { return x >= c0 && x < c0 + kBlock; }
  // stage state of any cell: shared memory when in the block, else SN + D
  __device__ __forceinline__ void state(int64_t x, float q[kNeqMax]) const {
    if (in_block(x)) {
      const int t = int(x - c0);
#pragma unroll
      for (int v = 0; v < kNeqMax; ++v) q[v] = v < ph.neq ? st[v][t] : 0.0f;
      return;
    }
    const int64_t n = a.n;
#pragma unroll
    for (int v = 0; v < kNeqMax; ++v) {
      if (v < ph.neq) {
        float s = __double2float_rn(__ldg(a.SN + v * n + x));
        if (a.Din) s += __ldg(a.Din + v * n + x);
        q[v] = s;
      } else {
        q[v] = 0.0f;
      }
    }
  }
  // neighbour value seen across face f of cell x (deltavalues.c): single
  // neighbour, mean of the 4 fine ones, or the boundary ghost
  __device__ __forceinline__ void across(int64_t x, int f, const float own[kNeqMax], float nb[kNeqMax]) const {
    const int32_t code = __ldg(a.nbr + f * a.n + x);
    if (code >= 0) {
      state(code, nb);
    } else if (is_hanging(code)) {
      const int32_t *k = a.hang_nbr + 4 * hang_index(code);
      float acc[kNeqMax] = {0.f, 0.f, 0.f, 0.f, 0.f};
      for (int s = 0; s < 4; ++s) {
        float q[kNeqMax];
        state(__ldg(k + s), q);
#pragma unroll
        for (int v = 0; v < kNeqMax; ++v) acc[v] += q[v];
      }
#pragma unroll
      for (int v = 0; v < kNeqMax; ++v) nb[v] = 0.25f * acc[v];
    } else {
      const int bc = -1 - code;
#pragma unroll
      for (int v = 0; v < kNeqMax; ++v) nb[v] = own[v];
      if (bc == 1 || bc == 3 || bc == 4) {
        FS g;
        mixed_face_state(ph, own, false, g);
        mixed_ghost(ph, bc, f, g);
#pragma unroll
        for (int v = 0; v < kNeqMax; ++v) nb[v] = g.q[v];
      }
    }
  }
  // MUSCL/minmod face value of face f of cell x (reconctruct_V3.c)
  __device__ __forceinline__ void recon_face(int64_t x, int32_t gx, int f, const float qx[kNeqMax],
                                             const float d0[kNeqMax], const float d1[kNeqMax],
                                             float out[kNeqMax]) const {
    const int lev = level_of(gx);
    const int rf = rel_of(gx, f), ro = rel_of(gx, opp_face(f));
    const float *gf = geo_face(a.geo, lev, f, rf);
    const float dcf = gf[0], inv_dcc_p = gf[1];
    const float inv_dcc_m = geo_face(a.geo, lev, opp_face(f), ro)[1];
#pragma unroll
    for (int v = 0; v < kNeqMax; ++v) {
      float grad = 0.0f;
      if (rf != kRelBoundary && fabsf(d0[v]) > 1e-10f) {
        const float sp = d0[v] * inv_dcc_p;
        const float sm = -d1[v] * inv_dcc_m;
        if (sm * sp > 0.0f) grad = fabsf(sm) > fabsf(sp) ? sp : sm;
      }
      out[v] = fmaf(dcf, grad, qx[v]);
    }
    (void)x;
  }
  // face value of face f of a cell outside the thread's own work (any cell)
  __device__ __forceinline__ void recon_any(int64_t x, int f, float out[kNeqMax]) const {
    float qx[kNeqMax], nbp[kNeqMax], nbm[kNeqMax], d0[kNeqMax], d1[kNeqMax];
    state(x, qx);
    across(x, f, qx, nbp);
    across(x, opp_face(f), qx, nbm);
#pragma unroll
    for (int v = 0; v < kNeqMax; ++v) {
      d0[v] = nbp[v] - qx[v];
      d1[v] = nbm[v] - qx[v];
    }
    recon_face(x, __ldg(a.geom + x), f, qx, d0, d1, out);
  }
};

// Block max of the per-cell FP32 CFL radius, folded into the FP64 maximum
// with an integer atomicMax on the bit pattern (exact and order-independent).
__device__ __forceinline__ void block_max_lambda_f(float lam, double *out) {
  __shared__ float red[kBlock / 32];
  for (int o = 16; o > 0; o >>= 1) lam = fmaxf(lam, __shfl_xor_sync(0xffffffffu, lam, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = lam;
  __syncthreads();
  if (threadIdx.x == 0) {
    float mx = red[0];
    for (int w = 1; w < kBlock / 32; ++w) mx = fmaxf(mx, red[w]);
    const double d = double(mx);
    if (d > 0.0 || isnan(d)) atomicMax((unsigned long long *)out, (unsigned long long)__double_as_longlong(d));
  }
}

// CFL spectral radius of one cell (definition in fvgpu.h), FP32.
__device__ __forceinline__ float cell_lambda_f(const MixedConst &mc, const GeoTables *geo, int32_t g,
                                               const float q[kNeqMax]) {
  const int lev = level_of(g);
  FS s;
  mixed_face_state(mc, q, false, s);
  float acc = 0.0f;
#pragma unroll
  for (int f = 0; f < 6; ++f) {
    const float un = fabsf(fmaf(s.w, mc.fr[9 * f + 2], fmaf(s.v, mc.fr[9 * f + 1], s.u * mc.fr[9 * f])));
    const int rel = rel_of(g, f);
    const float A = rel == kRelFiner ? 4.0f * geo->sub_area[lev * 6 + f] : geo_face(geo, lev, f, rel)[2];
    acc = fmaf(A, un + s.c, acc);
  }
  return acc * geo->inv2vol[lev];
}

__global__ void __launch_bounds__(kBlock) k_mixed_stage(MixedConst ph, StageArgs a) {
  __shared__ float st[kNeqMax][kBlock];
  __shared__ float sf[6][kNeqMax][kBlock];
  __shared__ float fp[3][kNeqMax][kBlock];
  const int t = threadIdx.x;
  const int64_t c0 = int64_t(blockIdx.x) * kBlock;
  const int64_t c = c0 + t;
  const int64_t n = a.n;
  const bool active = c < n;
  const int neq = ph.neq;
  const bool muscl = ph.ischeme == 2;
  Ctx cx(a, ph, c0, st);

  // A: own stage state
  double sn[kNeqMax];
  float din[kNeqMax], q[kNeqMax];
#pragma unroll
  for (int v = 0; v < kNeqMax; ++v) {
    sn[v] = 0.0;
    din[v] = 0.0f;
    q[v] = 0.0f;
    if (active && v < neq) {
      sn[v] = __ldg(a.SN + v * n + c);
      din[v] = a.Din ? __ldg(a.Din + v * n + c) : 0.0f;
      q[v] = __double2float_rn(sn[v]) + din[v];
    }
    st[v][t] = q[v];
  }
  int32_t nb[6];
  int32_t g = 0;
  if (active) {
    g = __ldg(a.geom + c);
#pragma unroll
    for (int f = 0; f < 6; ++f) nb[f] = __ldg(a.nbr + f * n + c);
  } else {
#pragma unroll
    for (int f = 0; f < 6; ++f) nb[f] = -3;
  }
  __syncthreads();

  // B: own face values
  if (active) {
    if (muscl) {
      float dl[6][kNeqMax];
#pragma unroll
      for (int f = 0; f < 6; ++f) {
        float nbv[kNeqMax];
        cx.across(c, f, q, nbv);
#pragma unroll
        for (int v = 0; v < kNeqMax; ++v) dl[f][v] = nbv[v] - q[v];
      }
#pragma unroll
      for (int f = 0; f < 6; ++f) {
        float o[kNeqMax];
        cx.recon_face(c, g, f, q, dl[f], dl[opp_face(f)], o);
#pragma unroll
        for (int v = 0; v < kNeqMax; ++v) sf[f][v][t] = o[v];
      }
    } else {
#pragma unroll
      for (int f = 0; f < 6; ++f)
#pragma unroll
        for (int v = 0; v < kNeqMax; ++v) sf[f][v][t] = q[v];
    }
  }
  __syncthreads();

  // face value of face f of cell x: shared memory when in the block
  auto face_value = [&](int64_t x, int f, float out[kNeqMax]) {
    if (cx.in_block(x)) {
      const int tx = int(x - c0);
#pragma unroll
      for (int v = 0; v < kNeqMax; ++v) out[v] = sf[f][v][tx];
    } else if (muscl) {
      cx.recon_any(x, f, out);
    } else {
      cx.state(x, out);
    }
  };

  // C: fluxes
  float R[kNeqMax] = {0.f, 0.f, 0.f, 0.f, 0.f};
  bool ok = true;
  const int lev = level_of(g);
  if (active) {
    // + faces: canonical lower cell is this one
#pragma unroll
    for (int f = 1; f < 6; ++f) {
      if (!is_plus_face(f)) continue;
      const int32_t code = nb[f];
      float own[kNeqMax];
#pragma unroll
      for (int v = 0; v < kNeqMax; ++v) own[v] = sf[f][v][t];
      FS L;
      ok &= mixed_face_state(ph, own, muscl, L);
      if (code >= 0 || is_boundary(code)) {
        FS Rs;
        int bc = 0;
        if (code >= 0) {
          float other[kNeqMax];
          face_value(code, opp_face(f), other);
          ok &= mixed_face_state(ph, other, muscl, Rs);
        } else {
          bc = -1 - code;
          Rs = L;
          mixed_ghost(ph, bc, f, Rs);
        }
        float Fn[kNeqMax];
        ok &= mixed_hllc_normal(ph, f, bc, L, Rs, Fn);
        const float A = geo_face(a.geo, lev, f, rel_of(g, f))[2];
#pragma unroll
        for (int v = 0; v < kNeqMax; ++v) {
          if (code >= 0) fp[plus_slot(f)][v][t] = Fn[v];
          R[v] -= A * Fn[v];
        }
      } else {  // 1:4 face: four sub-faces
        const int32_t *k = a.hang_nbr + 4 * hang_index(code);
        const float As = a.geo->sub_area[lev * 6 + f];
        for (int s = 0; s < 4; ++s) {
          float other[kNeqMax];
          face_value(__ldg(k + s), opp_face(f), other);
          FS Rs;
          ok &= mixed_face_state(ph, other, muscl, Rs);
          float Fn[kNeqMax];
          ok &= mixed_hllc_normal(ph, f, 0, L, Rs, Fn);
#pragma unroll
          for (int v = 0; v < kNeqMax; ++v) R[v] -= As * Fn[v];
        }
      }
    }
  }
  __syncthreads();
  if (active) {
    // - faces: canonical lower cell is the neighbour (or this cell at a boundary)
#pragma unroll
    for (int f = 0; f < 6; ++f) {
      if (is_plus_face(f)) continue;
      const int32_t code = nb[f];
      const int fo = opp_face(f);
      float own[kNeqMax];
#pragma unroll
      for (int v = 0; v < kNeqMax; ++v) own[v] = sf[f][v][t];
      if (is_boundary(code)) {
        FS Ls, Rs;
        ok &= mixed_face_state(ph, own, muscl, Ls);
        const int bc = -1 - code;
        Rs = Ls;
        mixed_ghost(ph, bc, f, Rs);
        float Fn[kNeqMax];
        ok &= mixed_hllc_normal(ph, f, bc, Ls, Rs, Fn);
        const float A = geo_face(a.geo, lev, f, kRelBoundary)[2];
#pragma unroll
        for (int v = 0; v < kNeqMax; ++v) R[v] -= A * Fn[v];
        continue;
      }
      const int rel = rel_of(g, f);
      if (code >= 0) {
        float Fn[kNeqMax];
        if (rel == kRelSame && cx.in_block(code)) {
          const int tl = int(code - c0);
#pragma unroll
          for (int v = 0; v < kNeqMax; ++v) Fn[v] = fp[plus_slot(fo)][v][tl];
        } else {
          // neighbour in another block, or coarser (its + face is a 1:4 face):
          // recompute the neighbour's canonical flux
          float lowv[kNeqMax];
          face_value(code, fo, lowv);
          FS Ls, Rs;
          ok &= mixed_face_state(ph, lowv, muscl, Ls);
          ok &= mixed_face_state(ph, own, muscl, Rs);
          ok &= mixed_hllc_normal(ph, fo, 0, Ls, Rs, Fn);
        }
        const float A = geo_face(a.geo, lev, f, rel)[2];
#pragma unroll
        for (int v = 0; v < kNeqMax; ++v) R[v] += A * Fn[v];
      } else {  // this cell is the coarse side of a 1:4 face on its - side
        const int32_t *k = a.hang_nbr + 4 * hang_index(code);
        const float As = a.geo->sub_area[lev * 6 + f];
        FS Rs;
        ok &= mixed_face_state(ph, own, muscl, Rs);
        for (int s = 0; s < 4; ++s) {
          const int64_t ks = __ldg(k + s);
          float Fn[kNeqMax];
          if (cx.in_block(ks)) {
            const int tl = int(ks - c0);
#pragma unroll
            for (int v = 0; v < kNeqMax; ++v) Fn[v] = fp[plus_slot(fo)][v][tl];
          } else {
            float lowv[kNeqMax];
            face_value(ks, fo, lowv);
            FS Ls;
            ok &= mixed_face_state(ph, lowv, muscl, Ls);
            ok &= mixed_hllc_normal(ph, fo, 0, Ls, Rs, Fn);
          }
#pragma unroll
          for (int v = 0; v < kNeqMax; ++v) R[v] += As * Fn[v];
        }
      }
    }
  }

  // D: RK stage in increment form, FP64 state at the last stage
  float lam = 0.0f;
  if (active) {
    bool finite = true;
#pragma unroll
    for (int v = 0; v < kNeqMax; ++v)
      if (v < neq && !isfinite(R[v])) finite = false;
    if (!ok) raise_error(a.err, kErrRegion, c);
    if (!finite) raise_error(a.err, kErrNonFinite, c);
    const float dtv = __double2float_rn(*a.dt) * a.geo->inv_vol[lev];
    float dn[kNeqMax];
#pragma unroll
    for (int v = 0; v < kNeqMax; ++v) {
      const float incr = dtv * R[v];
      switch (a.irk) {
        case 1: dn[v] = incr; break;
        case 2: dn[v] = 0.25f * (din[v] + incr); break;
        case 3: dn[v] = (2.0f / 3.0f) * (din[v] + incr); break;
        default: dn[v] = 0.5f * (din[v] + incr); break;
      }
    }
    if (a.last) {
      double snew[kNeqMax];
#pragma unroll
      for (int v = 0; v < kNeqMax; ++v) {
        if (v >= neq) break;
        snew[v] = sn[v] + double(dn[v]);
        a.SNout[v * n + c] = snew[v];
      }
      if (a.lambda) {
        // CFL spectral radius of the new state (FP32 per cell, max folded into FP64)
        float qn[kNeqMax];
#pragma unroll
        for (int v = 0; v < kNeqMax; ++v) qn[v] = v < neq ? __double2float_rn(snew[v]) : 0.0f;
        lam = cell_lambda_f(ph, a.geo, g, qn);
      }
    } else {
#pragma unroll
      for (int v = 0; v < kNeqMax; ++v)
        if (v < neq) a.Dout[v * n + c] = dn[v];
    }
  }
  if (a.last && a.lambda) block_max_lambda_f(lam, a.lambda);
}

// CFL radius of an FP64 state with the mixed geometry (first step).
__global__ void __launch_bounds__(kBlock) k_mixed_lambda(MixedConst ph, StageArgs a) {
  const int64_t c = int64_t(blockIdx.x) * kBlock + threadIdx.x;
  float lam = 0.0f;
  if (c < a.n) {
    float q[kNeqMax];
#pragma unroll
    for (int v = 0; v < kNeqMax; ++v) q[v] = v < ph.neq ? __double2float_rn(a.SN[v * a.n + c]) : 0.0f;
    lam = cell_lambda_f(ph, a.geo, __ldg(a.geom + c), q);
  }
  block_max_lambda_f(lam, a.lambda);
}

MixedConst make_const(const Phys &ph) {
  MixedConst mc;
  memset(&mc, 0, sizeof mc);
  for (int i = 0; i < 54; ++i) mc.fr[i] = float(ph.frames[i]);
  mc.gamma = float(ph.gamma);
  mc.pinf = float(ph.pinf);
  mc.gm1 = float(ph.gamma - 1.0);
  mc.gpinf = float(ph.gamma * ph.pinf);
  mc.ylo = float(ph.ymin / 1000.0);
  mc.yhi = float(1.0 - ph.ymin / 1000.0);
  for (int v = 0; v < kNeqMax; ++v) mc.inflow[v] = float(ph.inflow[v]);
  mc.model = ph.model;
  mc.neq = ph.neq;
  mc.ischeme = ph.ischeme;
  return mc;
}

// resource slots
enum { kBufGeom = 0, kBufTables = 1, kBufD1 = 2, kBufD2 = 3, kBufAlt = 4 };

cudaError_t alloc_slot(MixedResources &r, int slot, size_t bytes) {
  if (r.buf[slot]) cudaFree(r.buf[slot]);
  r.buf[slot] = nullptr;
  r.bytes[slot] = 0;
  cudaError_t e = cudaMalloc(&r.buf[slot], bytes ? bytes : 16);
  if (e == cudaSuccess) r.bytes[slot] = bytes;
  return e;
}

}  // namespace

bool mixed_supported(const Phys &ph, char *why, size_t whylen) {
  if (ph.model != 1 && ph.model != 3) {
    snprintf(why, whylen, "the mixed path implements models 1 and 3");
    return false;
  }
  if (ph.ns != 0) {
    snprintf(why, whylen, "the mixed path does not implement viscous fluxes (use FVGPU_FP64)");
    return false;
  }
  return true;
}

int mixed_prepare_host(MixedResources &r, const Phys &ph, const fvgpu_mesh_soa *m, char *why, size_t whylen) {
  r.ready = false;
  char tmp[256];
  if (!mixed_supported(ph, tmp, sizeof tmp)) {
    snprintf(why, whylen, "%s", tmp);
    return FVGPU_ERR_UNSUPPORTED;
  }
  if (!m->level) {
    snprintf(why, whylen, "the mixed path needs the per-cell level array");
    return FVGPU_ERR_UNSUPPORTED;
  }
  // + faces must carry +x, +y, +z normals and each face its opposite's negation
  static const int axis[6] = {1, 0, 1, 0, 2, 2};
  for (int f = 0; f < 6; ++f) {
    for (int k = 0; k < 3; ++k) {
      const double nk = m->frames[9 * f + k];
      const double want = k == axis[f] ? (is_plus_face(f) ? 1.0 : -1.0) : 0.0;
      if (nk != want) {
        snprintf(why, whylen, "the mixed path needs axis-aligned face frames (face %d)", f);
        return FVGPU_ERR_UNSUPPORTED;
      }
    }
  }
  const int64_t n = m->ncells;
  GeoTables gt;
  memset(&gt, 0, sizeof gt);
  std::vector<char> seen(kGeoEntries, 0), seen_sub((kMaxLevel + 1) * 6, 0), seen_vol(kMaxLevel + 1, 0);
  std::vector<int32_t> geom(size_t(n), 0);
  for (int64_t c = 0; c < n; ++c) {
    const int lev = m->level[c];
    if (lev < 0 || lev > kMaxLevel) {
      snprintf(why, whylen, "cell %lld: level %d outside 0..%d", (long long)c, lev, kMaxLevel);
      return FVGPU_ERR_UNSUPPORTED;
    }
    int32_t code = lev;
    if (!seen_vol[lev]) {
      seen_vol[lev] = 1;
      gt.vol[lev] = float(m->vol[c]);
      gt.inv_vol[lev] = float(1.0 / m->vol[c]);
      gt.inv2vol[lev] = float(1.0 / (2.0 * m->vol[c]));
    } else if (gt.vol[lev] != float(m->vol[c]) || gt.inv_vol[lev] != float(1.0 / m->vol[c])) {
      snprintf(why, whylen, "the mixed path needs one volume per level (cell %lld)", (long long)c);
      return FVGPU_ERR_UNSUPPORTED;
    }
    for (int f = 0; f < 6; ++f) {
      const int64_t i = f * n + c;
      const int32_t nc = m->nbr[i];
      int rel;
      if (nc < 0 && nc > FVGPU_HANG0) {
        rel = kRelBoundary;
      } else if (nc <= FVGPU_HANG0) {
        rel = kRelFiner;
        const int64_t h = int64_t(FVGPU_HANG0) - nc;
        const float sa = float(m->hang_area[4 * h]);
        for (int s = 1; s < 4; ++s)
          if (float(m->hang_area[4 * h + s]) != sa) {
            snprintf(why, whylen, "the mixed path needs equal sub-face areas");
            return FVGPU_ERR_UNSUPPORTED;
          }
        const int k = lev * 6 + f;
        if (!seen_sub[k]) {
          seen_sub[k] = 1;
          gt.sub_area[k] = sa;
        } else if (gt.sub_area[k] != sa) {
          snprintf(why, whylen, "the mixed path needs one sub-face area per level and face");
          return FVGPU_ERR_UNSUPPORTED;
        }
      } else {
        const int nl = m->level[nc];
        if (nl == lev)
          rel = kRelSame;
        else if (nl == lev - 1)
          rel = kRelCoarser;
        else {
          snprintf(why, whylen, "cell %lld face %d: neighbour level %d", (long long)c, f, nl);
          return FVGPU_ERR_UNSUPPORTED;
        }
        if (m->nbr_face[i] != opp_face(f)) {
          snprintf(why, whylen, "the mixed path needs neighbour face = opposite face");
          return FVGPU_ERR_UNSUPPORTED;
        }
      }
      code |= rel << (5 + 2 * f);
      const float dcf = float(m->dcf[i]);
      const float inv_dcc = m->dcc[i] > 0.0 ? float(1.0 / m->dcc[i]) : __builtin_inff();
      const float area = rel == kRelFiner ? 0.0f : float(m->area[i]);
      const int gi = geo_index(lev, f, rel);
      float *e = gt.face + gi * kGeoStride;
      if (!seen[gi]) {
        seen[gi] = 1;
        e[0] = dcf;
        e[1] = inv_dcc;
        e[2] = area;
      } else if (e[0] != dcf || !(e[1] == inv_dcc) || e[2] != area) {
        snprintf(why, whylen, "the mixed path needs octree-regular geometry (cell %lld face %d)", (long long)c, f);
        return FVGPU_ERR_UNSUPPORTED;
      }
    }
    geom[size_t(c)] = code;
  }
  cudaError_t e;
  if ((e = alloc_slot(r, kBufGeom, sizeof(int32_t) * n)) != cudaSuccess ||
      (e = cudaMemcpy(r.buf[kBufGeom], geom.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = alloc_slot(r, kBufTables, sizeof(GeoTables))) != cudaSuccess ||
      (e = cudaMemcpy(r.buf[kBufTables], &gt, sizeof gt, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = alloc_slot(r, kBufD1, sizeof(float) * kNeqMax * n)) != cudaSuccess ||
      (e = alloc_slot(r, kBufD2, sizeof(float) * kNeqMax * n)) != cudaSuccess ||
      (e = alloc_slot(r, kBufAlt, sizeof(double) * kNeqMax * n)) != cudaSuccess) {
    snprintf(why, whylen, "mixed-path allocation: %s", cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? FVGPU_ERR_NOMEM : FVGPU_ERR_CUDA;
  }
  r.n = n;
  r.ready = true;
  return FVGPU_OK;
}

void release_mixed(MixedResources &r) {
  for (int i = 0; i < 8; ++i) {
    if (r.buf[i]) cudaFree(r.buf[i]);
    r.buf[i] = nullptr;
    r.bytes[i] = 0;
  }
  r.ready = false;
}

static StageArgs stage_args(MixedResources &r, const MeshView &m) {
  StageArgs a{};
  a.n = m.n;
  a.nbr = m.nbr;
  a.geom = static_cast<const int32_t *>(r.buf[kBufGeom]);
  a.hang_nbr = m.hang_nbr;
  a.geo = static_cast<const GeoTables *>(r.buf[kBufTables]);
  return a;
}

double *mixed_alt_state(MixedResources &r) { return static_cast<double *>(r.buf[kBufAlt]); }

void mixed_swap_state(MixedResources &r, void *&state) {
  void *t = state;
  state = r.buf[kBufAlt];
  r.buf[kBufAlt] = t;
}

cudaError_t enqueue_mixed_lambda(MixedResources &r, const Phys &ph, const MeshView &m, const double *S,
                                 double *lambda, LaunchMarks &marks, cudaStream_t st) {
  StageArgs a = stage_args(r, m);
  a.SN = S;
  a.lambda = lambda;
  marks.mark(FVGPU_KIND_DT);
  k_mixed_lambda<<<unsigned((m.n + kBlock - 1) / kBlock), kBlock, 0, st>>>(make_const(ph), a);
  return cudaGetLastError();
}

// One RK step from state `in` to state `out` (out != in).
cudaError_t enqueue_step_mixed(MixedResources &r, const Phys &ph, const MeshView &m, int scheme, bool cfl_mode,
                               const double *in, double *out, double *dt, double *lambda, const double *cfl,
                               unsigned long long *err, LaunchMarks &marks, cudaStream_t st) {
  static const int kStages[4][3] = {{0, 0, 0}, {1, 0, 0}, {1, 4, 0}, {1, 2, 3}};
  const int nst = scheme == 1 ? 1 : (scheme == 2 ? 2 : 3);
  if (cfl_mode) {
    marks.mark(FVGPU_KIND_DT);
    launch_dt_from_lambda(lambda, lambda, cfl, dt, err, st);
  }
  float *D[2] = {static_cast<float *>(r.buf[kBufD1]), static_cast<float *>(r.buf[kBufD2])};
  const MixedConst mc = make_const(ph);
  const unsigned grid = unsigned((m.n + kBlock - 1) / kBlock);
  for (int k = 0; k < nst; ++k) {
    StageArgs a = stage_args(r, m);
    a.SN = in;
    a.Din = k == 0 ? nullptr : D[(k - 1) & 1];
    a.Dout = D[k & 1];
    a.SNout = out;
    a.dt = dt;
    a.irk = kStages[scheme][k];
    a.last = k == nst - 1;
    a.lambda = (a.last && cfl_mode) ? lambda : nullptr;
    a.err = err;
    marks.mark(FVGPU_KIND_MIXED_STAGE);
    k_mixed_stage<<<grid, kBlock, 0, st>>>(mc, a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace fv
