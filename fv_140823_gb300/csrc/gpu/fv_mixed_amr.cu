// fvbuild: -fmad=false
//
// FP32-mixed path, table-driven kernel family: every mesh that is not model
// 1 in 8x8x4 bricks throughout (AMR meshes with 1:4 faces, meshes whose
// same-level blocks are 4x4x4 or smaller, model 3, FVGPU_FLAG_NO_BRICKS).
// fv_mixed.cu holds the slope-sharing brick kernel of uniform model-1 meshes
// and chooses the family when a mesh is prepared; a context runs one family
// throughout, so its results do not depend on how its cells are split into
// blocks.  This family evaluates each face value per face (reconctruct_V3.c)
// and sums a cell's residual face by face.
//
// Arithmetic.  Reconstruction, equation of state and HLLC fluxes run in FP32
// (model 3's paired density words, their reconstruction and the mixture EOS
// pressure inversion in float-float, 48 bits).  The state is kept in FP64
// as the step-start state SN; a stage carries only the FP32 increment
// D_k = S_k - SN, so the RK stage formulas of RK.c become
//     RK(1): D1 = dt/V R(S0)                  (S1 = SN + dt/V R)
//     RK(2): D2 = 1/4 (D1 + dt/V R(S1))       (S2 = 3/4 SN + 1/4 S1 + 1/4 dt/V R)
//     RK(3): D3 = 2/3 (D2 + dt/V R(S2))       (S3 = 1/3 SN + 2/3 S2 + 2/3 dt/V R)
//     RK(4): D  = 1/2 (D1 + dt/V R(S1))       (SSP-RK2 second stage)
// and each step ends with one FP64 add per variable, SN <- SN + D_last, plus
// an FP32 copy SNf of the new state that the next step's stages read.  On
// GB300 FP64 adds and multiplies run at ~1/70 of the FP32 rate (measured:
// 0.51 against 37 T thread-ops/s), so the stages touch no FP64 value except
// at the last one: the per-stage increments are small against the state,
// their FP32 rounding is ~1e-8 of the state per stage, and every add into
// the state is FP64.
//
// Canonical face fluxes.  Every face flux is defined from the face's lower
// cell (the one whose +x/+y/+z face it is), with that face's frame; the
// lower cell's residual gets -A F and the upper cell's +A F.  Whoever
// evaluates a face gets the same bits (this translation unit is compiled
// without automatic multiply-add contraction, explicit fmaf only), so the
// scheme is conservative and deterministic however the work is split.
//
// Face frames are those of the reference's hexahedral cells (checked at
// upload), compiled in as signed permutations: rotating the momentum into
// and out of a face frame is a choice of registers.
//
// Two kernels share that definition:
//   k_mixed_brick    a Morton-aligned 8x8x4 (or, on AMR meshes, 4x4x4)
//                    brick of same-level cells whose six sides are same-level
//                    blocks of that shape or domain boundaries: brick +
//                    2-deep face halo staged in shared memory through
//                    constant index tables, every face of the brick
//                    evaluated once (a brick off the domain boundary: each
//                    thread its cell's +x, +y, +z faces, then the first
//                    threads the faces on the brick's lower sides), no
//                    neighbour tables read; viscous runs (model 1) read the
//                    two cells' gradients of each face;
//   k_mixed_general  any other run of up to 256 consecutive cells (AMR
//                    interfaces, 1:4 faces): table-driven, each thread
//                    computes its + faces and publishes them, the upper cell
//                    reuses them or recomputes the canonical flux across
//                    block edges and 1:4 sub-faces.
// A cell's residual is accumulated in the same face order with the same
// operations in both kernels, so its result does not depend on which kernel
// handled it (tests compare the two bit for bit).
//
// Geometry comes from per-level tables (octree-regular meshes): a packed
// per-cell code (level + face relations) replaces the FP64 face tables.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <vector>

#include "fv_mixed.cuh"

namespace fv {
namespace amr {

namespace {

constexpr int kBlock = 256;
constexpr int kMaxLevel = 18;
constexpr int kRelSame = 0, kRelFiner = 1, kRelCoarser = 2, kRelBoundary = 3;
constexpr int kGeoStride = 4;  // per (level, face, relation): dcf, 1/dcc, area, pad
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
__device__ __forceinline__ int plus_slot(int f) { return f == 1 ? 0 : (f == 2 ? 1 : 2); }
// residual accumulation order (both kernels): +x, +y, +z, -x, -y, -z
__device__ __forceinline__ int face_of_iter(int it) {
  return it == 0 ? 1 : it == 1 ? 2 : it == 2 ? 5 : it == 3 ? 3 : it == 4 ? 0 : 4;
}

// FP32 constants, converted once on the host.
struct MixedConst {
  float fr[54];  // face frames n, t1, t2 per face index
  float gamma, pinf, gm1, gpinf;
  float ylo, yhi;  // mass-fraction clip (facercnstr.c:43-44)
  float visc;      // dynamic viscosity (flux_viscous.c, turb = 0)
  int ns, eos;     // viscous fluxes on; energy work term on
  float inflow[7];  // state words of the inflow ghost (model 3: seven)
  int model, neq, ischeme, pad;
};

// A block of work: a brick (type 0) or a general run (type 1).
struct BlockDesc {
  int start;    // first cell
  int count;    // cells (256 for a brick)
  int level;    // brick level
  int side[6];  // brick side per face index: >= 0 first cell of the neighbour brick, < 0: -1 - bc
  int pad;
};

struct StageArgs {
  int n;
  const int32_t *nbr;       // [6][n]
  const int32_t *geom;      // [n]: level | rel_f << (5 + 2 f)
  const int32_t *hang_nbr;  // [nhang][4]
  const GeoTables *geo;
  const BlockDesc *blocks;
  const float *SNf;         // [neq][n] FP32 copy of the step-start state
  const float *Sin;         // [neq][n] FP32 stage-input state SNf + Din (SNf at the first stage)
  const float *Din;         // [neq][n] stage-input increment (null: zero)
  float *Dout;              // [neq][n]
  float *Sout;              // [neq][n] non-last stages: the next stage's input SNf + Dout
  const float *SG;          // [9][n] viscous runs: momentum gradients of Sin (ux uy uz vx ... wz)
  const double *SN;         // [neq][n] step-start state (last stage)
  double *SNout;            // [neq][n] last stage: SN + D
  float *SNfout;            // [neq][n] last stage: FP32 copy of SNout
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

struct FS {
  float r, u, v, w, e, p, c, y;
};

__device__ __forceinline__ float fast_rcp(float x) { return __fdividef(1.0f, x); }
__device__ __forceinline__ float fast_sqrt(float x) { return x == 0.0f ? 0.0f : x * rsqrtf(x); }

// State words.  Model 1 keeps its five conservative variables as FP32
// words.  Model 3 (liquid-gas mixture) keeps the density and the gas partial
// density rho Y as pairs of FP32 words, a high word and the rounding
// remainder (words 0 + 5 and 4 + 6), with the density shifted by kRhoOff, the
// saturation density of the mixture EOS (barotropic_eos.c:41, as an FP32
// value).  The pressure inversion is stiff in both partial densities: near
// the liquid density an FP32 ulp of rho is 6e-5, which the liquid branch
// (dp/drho = c_liq^2) turns into ~130 Pa, and the gas density (~1) stored as
// rho - kRhoOff alone would carry the ulp of ~1000, ~5 Pa of gas pressure.
// With the pairs, model 3's reconstruction of rho and rho Y (differences,
// limited slopes, face values) and the pressure inversion run in float-float
// arithmetic (48 bits, below) and see the face values to that rounding; the
// momentum and the flux arithmetic stay FP32.  Stage increments stay five
// FP32 words.  FP64 remains where the FP64 state is read or written (the
// last stage's update, the conversion of an uploaded state).
template <int MODEL>
constexpr int kNv = MODEL == 3 ? 7 : 5;
constexpr int kNvMax = 7;
constexpr float kRhoOffF = 998.1618f;
constexpr double kRhoOffD = double(kRhoOffF);
// the low word of paired variable v (0: the density, 4: rho Y)
__host__ __device__ constexpr int lo_word(int v) { return v == 0 ? 5 : 6; }

// Float-float arithmetic on the FP32 pipe.  A value is the unevaluated sum
// hi + lo of two floats with |lo| <= ulp(hi) / 2 -- exactly the form of a
// paired word -- so it carries 48 significant bits.  Error-free steps:
// Knuth's two-sum, Dekker's fast two-sum (|a| >= |b|), and the exact product
// a*b - p by one fused multiply-add; sums and products of two pairs are the
// usual double-single forms (error about 2^-46 of the operands).  GB300's
// FP64 pipe issues at a small fraction of the FP32 rate, so model 3 keeps its
// paired words, their reconstruction and the pressure inversion here and
// uses FP64 only where the FP64 state is read or written.  This file is built
// with -fmad=false, so no product is fused into a two-sum.
struct FF {
  float hi, lo;
};
__device__ __forceinline__ FF ff_fast_two_sum(float a, float b) {
  const float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ FF ff_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  const FF s = ff_two_sum(a.hi, b.hi);
  return ff_fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
__device__ __forceinline__ FF ff_neg(FF a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ FF ff_sub(FF a, FF b) { return ff_add(a, ff_neg(b)); }
__device__ __forceinline__ FF ff_mul_f(FF a, float b) {
  const float p = a.hi * b;
  return ff_fast_two_sum(p, fmaf(a.lo, b, fmaf(a.hi, b, -p)));
}
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
  const float p = a.hi * b.hi;
  return ff_fast_two_sum(p, fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, fmaf(a.hi, b.hi, -p))));
}
// square root of a >= 0: the FP32 root and one Newton step on the pair
__device__ __forceinline__ FF ff_sqrt(FF a) {
  if (!(a.hi > 0.0f)) return {0.0f, 0.0f};
  const float s = __fsqrt_rn(a.hi);
  const FF r = ff_sub(a, FF{s * s, fmaf(s, s, -(s * s))});
  return ff_fast_two_sum(s, __fdiv_rn(r.hi, 2.0f * s));
}
__device__ __forceinline__ FF ff_abs(FF a) { return a.hi < 0.0f ? ff_neg(a) : a; }
// a FP64 constant as a pair (host or device)
__host__ __device__ constexpr FF ff_const(double x) { return {float(x), float(x - double(float(x)))}; }
// paired word v as a pair, and a pair stored as paired word v
__device__ __forceinline__ FF pair_ff(const float *q, int v) { return {q[v], q[lo_word(v)]}; }
__device__ __forceinline__ void set_pair_ff(float *q, int v, FF x) {
  q[v] = x.hi;
  q[lo_word(v)] = x.lo;
}
// the density of a model-3 state as a pair (its offset added back)
__device__ __forceinline__ FF state_rho_ff(const float *q) { return ff_add(FF{kRhoOffF, 0.0f}, pair_ff(q, 0)); }
// splits an FP64 value into paired word v
__device__ __forceinline__ void set_pair(float *q, int v, double x) {
  const float h = __double2float_rn(x);
  q[v] = h;
  q[lo_word(v)] = __double2float_rn(x - double(h));
}
// the density in FP32
template <int MODEL>
__device__ __forceinline__ float state_rho(const float *q) {
  if constexpr (MODEL == 3) return state_rho_ff(q).hi;
  return q[0];
}
// FP32 state words of an FP64 state (model 3: seven words)
template <int MODEL>
__device__ __forceinline__ void to_state_words(const double x[kNeqMax], float q[kNvMax]) {
#pragma unroll
  for (int v = 0; v < kNeqMax; ++v) q[v] = __double2float_rn(x[v]);
  if constexpr (MODEL == 3) {
    set_pair(q, 0, x[0] - kRhoOffD);
    set_pair(q, 4, x[4]);
  }
}

// The two-phase mixture EOS of barotropic_eos.c:32-129 (the larger root of
// the pressure quadratic, the liquid sound speed with the mixture fallback)
// on the two partial densities: the reference's products rho Y and
// rho (1 - Y) are the gas partial density ry and rho - ry, taken as such from
// the paired state words.  Float-float: b = c^2 r_sat - p_sat - ry R T -
// (rho - ry) c^2 cancels to a few parts in 1e4 of its terms in the liquid, and
// the pairs keep it to ~1e-10 of the pressure.  The larger root is returned
// rounded to FP32; false when neither branch has a real root.
// one branch of the inversion: sound speed squared c2 (exact in FP32), k1 =
// c^2 r_sat - p_sat, k2 = p_sat - c^2 r_sat; false without a real root
__device__ __forceinline__ bool mixture_root(FF rg, FF rl, FF k1, FF k2, float c2, float &p) {
  const FF b = ff_sub(ff_sub(k1, rg), ff_mul_f(rl, c2));
  const FF d = ff_mul(k2, rg);
  const FF disc = ff_sub(ff_mul(b, b), ff_mul_f(d, 4.0f));
  if (!(disc.hi >= 0.0f)) return false;
  p = ff_mul_f(ff_sub(ff_sqrt(disc), b), 0.5f).hi;
  return true;
}
__device__ __forceinline__ bool eos_mixture_ff(FF r, FF ry, float &p_out, float &c_out) {
  constexpr double R_G = 286.0, T_ref = 293.15, r_sat = 998.1618, p_sat = 2340.0;
  constexpr double c_liq = 1482.5, c_mix = 1.0;
  constexpr FF kRT = ff_const(R_G * T_ref);
  const FF rg = ff_mul(ry, kRT), rl = ff_sub(r, ry);
  c_out = float(c_liq);
  if (mixture_root(rg, rl, ff_const(c_liq * c_liq * r_sat - p_sat), ff_const(p_sat - c_liq * c_liq * r_sat),
                   float(c_liq * c_liq), p_out))
    return true;
  c_out = float(c_mix);
  if (mixture_root(rg, rl, ff_const(c_mix * c_mix * r_sat - p_sat), ff_const(p_sat - c_mix * c_mix * r_sat),
                   float(c_mix * c_mix), p_out))
    return true;
  p_out = __int_as_float(0x7fc00000);
  return false;
}

// Model 3: the density and gas partial density of a face value as pairs for
// the pressure inversion, with the mass fraction clipped as
// facercnstr.c:43-44 (clip), and returned in FP32 for the flux.
__device__ __forceinline__ bool mixture_face_eos(const MixedConst &mc, const float *q, bool clip, float &r32,
                                                 float &y32, float &p32, float &c32) {
  const FF r = state_rho_ff(q);
  FF ry = pair_ff(q, 4);
  r32 = r.hi;
  y32 = ry.hi * fast_rcp(r32);
  if (clip && (y32 < mc.ylo || y32 > mc.yhi)) {
    y32 = y32 < mc.ylo ? mc.ylo : mc.yhi;
    ry = ff_mul_f(r, y32);
  }
  return eos_mixture_ff(r, ry, p32, c32);
}

// FP32 face state (facercnstr.c:20-59 / facevalues.c:113-142).
template <int MODEL>
__device__ __forceinline__ bool mixed_face_state(const MixedConst &mc, const float *q, bool clip, FS &s) {
  if (MODEL == 1) {
    s.r = q[0];
    const float rinv = fast_rcp(s.r);
    s.u = q[1] * rinv;
    s.v = q[2] * rinv;
    s.w = q[3] * rinv;
    s.e = q[4];
    const float ke = fmaf(s.w, s.w, fmaf(s.v, s.v, s.u * s.u));
    const float e_int = fmaf(-0.5f, ke, s.e * rinv);
    s.p = fmaf(s.r * mc.gm1, e_int, -mc.gpinf);
    s.c = fast_sqrt(mc.gamma * (s.p + mc.pinf) * rinv);
    s.y = 0.0f;
    return true;
  }
  // model 3: pressure inversion in float-float on the paired words
  const bool ok = mixture_face_eos(mc, q, clip, s.r, s.y, s.p, s.c);
  const float rinv = fast_rcp(s.r);
  s.u = q[1] * rinv;
  s.v = q[2] * rinv;
  s.w = q[3] * rinv;
  s.e = 0.0f;
  return ok;
}

// Value across a boundary face (deltavalues.c:9-14; bc.c:19-49): the own
// state (transmissive), the inflow state, or the own state with the momentum
// mirrored as such (slip wall: normal component; no-slip wall: all of it),
// which on the axis-aligned faces is exact, as in the FP64 path.
template <int MODEL>
__device__ __forceinline__ void boundary_value(const MixedConst &mc, int bc, int f, const float *own, float *nb) {
#pragma unroll
  for (int v = 0; v < kNv<MODEL>; ++v) nb[v] = own[v];
  if (bc == 1) {
#pragma unroll
    for (int v = 0; v < kNv<MODEL>; ++v) nb[v] = mc.inflow[v];
  } else if (bc == 3) {
    const float nx = mc.fr[9 * f], ny = mc.fr[9 * f + 1], nz = mc.fr[9 * f + 2];
    const float mn = fmaf(own[3], nz, fmaf(own[2], ny, own[1] * nx));
    nb[1] = fmaf(-2.0f * mn, nx, own[1]);
    nb[2] = fmaf(-2.0f * mn, ny, own[2]);
    nb[3] = fmaf(-2.0f * mn, nz, own[3]);
  } else if (bc == 4) {
    nb[1] = -own[1];
    nb[2] = -own[2];
    nb[3] = -own[3];
  }
}

// Face-local state: the momentum rotated into the face frame (normal n,
// tangents t1, t2), its velocities, pressure and sound speed.  The mixed
// path requires orthonormal frames (checked at upload), so the kinetic energy
// and the stress contraction n.(p I).n = p are frame invariant.
struct LS {
  float r, mn, mm, ml, q4;  // density, local momentum, fifth conservative variable
  float un, um, ul;         // local velocity
  float p, c, e, y;
};

// Face frames of the reference's hexahedral cells (tagvector.c:40-53 on
// axis-aligned cells; the mixed path requires them, checked at upload): n,
// t1, t2 per face index.  Every row has one nonzero entry, +-1, so rotating
// into and out of a face frame is a signed permutation of the components:
// exact, and the same bits whether the face index is known at compile time
// (brick faces) or only at run time.
__host__ __device__ constexpr float std_frame(int f, int k) {
  constexpr float t[6][9] = {{0, -1, 0, 1, 0, 0, 0, 0, 1},  {1, 0, 0, 0, 0, 1, 0, -1, 0},
                             {0, 1, 0, 0, 0, 1, 1, 0, 0},   {-1, 0, 0, 0, -1, 0, 0, 0, 1},
                             {0, 0, -1, 1, 0, 0, 0, -1, 0}, {0, 0, 1, 0, -1, 0, 1, 0, 0}};
  return t[f][k];
}
// column of the nonzero entry of row r of frame f; row whose nonzero entry
// is in column k; sign of row r (compile-time use only)
__host__ __device__ constexpr int frame_col(int f, int r) {
  return std_frame(f, 3 * r) != 0.0f ? 0 : (std_frame(f, 3 * r + 1) != 0.0f ? 1 : 2);
}
__host__ __device__ constexpr int frame_row(int f, int k) {
  return std_frame(f, k) != 0.0f ? 0 : (std_frame(f, 3 + k) != 0.0f ? 1 : 2);
}
__host__ __device__ constexpr bool frame_neg(int f, int r) { return std_frame(f, 3 * r + frame_col(f, r)) < 0.0f; }

template <int F, int R>
__device__ __forceinline__ float frame_in_row(const float q[kNeqMax]) {
  constexpr int k = frame_col(F, R);
  constexpr bool neg = frame_neg(F, R);
  return neg ? -q[1 + k] : q[1 + k];
}
template <int F, int K>
__device__ __forceinline__ float frame_out_col(float a, float b, float c) {
  constexpr int r = frame_row(F, K);
  constexpr bool neg = frame_neg(F, r);
  const float x = r == 0 ? a : (r == 1 ? b : c);
  return neg ? -x : x;
}
template <int F>
__device__ __forceinline__ void frame_in_f(const float q[kNeqMax], float &mn, float &mm, float &ml) {
  mn = frame_in_row<F, 0>(q);
  mm = frame_in_row<F, 1>(q);
  ml = frame_in_row<F, 2>(q);
}
template <int F>
__device__ __forceinline__ void frame_out_f(float a, float b, float c, float out[kNeqMax]) {
  out[1] = frame_out_col<F, 0>(a, b, c);
  out[2] = frame_out_col<F, 1>(a, b, c);
  out[3] = frame_out_col<F, 2>(a, b, c);
}
// momentum into the frame of face F (F < 0: face f, known at run time)
template <int F>
__device__ __forceinline__ void frame_in(int f, const float q[kNeqMax], float &mn, float &mm, float &ml) {
  if constexpr (F >= 0) {
    frame_in_f<F>(q, mn, mm, ml);
  } else {
    switch (f) {
      case 0: frame_in_f<0>(q, mn, mm, ml); break;
      case 1: frame_in_f<1>(q, mn, mm, ml); break;
      case 2: frame_in_f<2>(q, mn, mm, ml); break;
      case 3: frame_in_f<3>(q, mn, mm, ml); break;
      case 4: frame_in_f<4>(q, mn, mm, ml); break;
      default: frame_in_f<5>(q, mn, mm, ml); break;
    }
  }
}
// face-frame momentum components (a, b, c) back to out[1..3]
template <int F>
__device__ __forceinline__ void frame_out(int f, float a, float b, float c, float out[kNeqMax]) {
  if constexpr (F >= 0) {
    frame_out_f<F>(a, b, c, out);
  } else {
    switch (f) {
      case 0: frame_out_f<0>(a, b, c, out); break;
      case 1: frame_out_f<1>(a, b, c, out); break;
      case 2: frame_out_f<2>(a, b, c, out); break;
      case 3: frame_out_f<3>(a, b, c, out); break;
      case 4: frame_out_f<4>(a, b, c, out); break;
      default: frame_out_f<5>(a, b, c, out); break;
    }
  }
}

template <int MODEL, int F = -1>
__device__ __forceinline__ bool local_state(const MixedConst &mc, int f, const float *q, bool clip, LS &s) {
  if (MODEL == 1) {
    s.r = q[0];
    s.q4 = q[4];
    frame_in<F>(f, q, s.mn, s.mm, s.ml);
    const float rinv = fast_rcp(s.r);
    s.un = s.mn * rinv;
    s.um = s.mm * rinv;
    s.ul = s.ml * rinv;
    s.e = q[4];
    s.y = 0.0f;
    // p = (gamma - 1) (E - rho |u|^2 / 2) - gamma pinf, rho |u|^2 as m . u
    const float ke2 = fmaf(s.ml, s.ul, fmaf(s.mm, s.um, s.mn * s.un));
    s.p = fmaf(mc.gm1, fmaf(-0.5f, ke2, s.e), -mc.gpinf);
    s.c = fast_sqrt(mc.gamma * (s.p + mc.pinf) * rinv);
    return true;
  }
  // model 3: pressure inversion in float-float on the paired words
  const bool ok = mixture_face_eos(mc, q, clip, s.r, s.y, s.p, s.c);
  s.q4 = q[4];
  frame_in<F>(f, q, s.mn, s.mm, s.ml);
  const float rinv = fast_rcp(s.r);
  s.un = s.mn * rinv;
  s.um = s.mm * rinv;
  s.ul = s.ml * rinv;
  s.e = 0.0f;
  return ok;
}

// Ghost of a boundary face in the face-local frame (bc.c:19-49): inflow
// state, transmissive copy, slip wall (normal velocity mirrored), no-slip
// wall (velocity reversed).
template <int MODEL, int F = -1>
__device__ __forceinline__ void local_ghost(const MixedConst &mc, int bc, int f, LS &g) {
  if (bc == 1) {
    local_state<MODEL, F>(mc, f, mc.inflow, false, g);
  } else if (bc == 3 || bc == 4) {
    g.un = -g.un;
    g.mn = -g.mn;
    if (bc == 4) {
      g.um = -g.um;
      g.ul = -g.ul;
      g.mm = -g.mm;
      g.ml = -g.ml;
    }
  }
}

// HLLC normal flux F.n + S_K (U*_K - U_K) through a face of frame f
// (hllc_euler.c:3-55, compute_wave_speeds.c:3-88, star_region_euler.c:3-40,
// contracted with n as residual_faces_AMR.c:145-149), evaluated in the face
// frame and rotated back once.
template <int MODEL, int F = -1>
__device__ __forceinline__ bool local_hllc(const MixedConst &mc, int f, int bc, const LS &L, const LS &R,
                                           float Fn[kNeqMax]) {
  const float SR = fmaxf(L.un + L.c, R.un + R.c);
  const float SL = fminf(L.un - L.c, R.un - R.c);
  const float num = fmaf(SR, R.mn, fmaf(-SL, L.mn, fmaf(L.mn, L.un, L.p) - fmaf(R.mn, R.un, R.p)));
  const float den = fmaf(SR, R.r, fmaf(-SL, L.r, L.mn - R.mn));
  float S_S = __fdividef(num, den);
  const bool ok = !isnan(S_S);
  if (bc == 3) S_S = 0.0f;
  // region selection of hllc_euler.c:18-50 (0 <= SL: left; SL <= 0 <= S*:
  // left star; S* <= 0 <= SR: right star; SR <= 0: right), reduced to two
  // predicates; with S* not NaN (NaN wave speeds make S* NaN) exactly one
  // region holds
  const bool gl = 0.0f <= SL, gs = 0.0f <= S_S, gr = 0.0f <= SR;
  const bool left = gl || gs;
  const bool star = !gl && (gs || gr);
  const float Kr = left ? L.r : R.r, Kmn = left ? L.mn : R.mn;
  const float Kun = left ? L.un : R.un, Kum = left ? L.um : R.um, Kul = left ? L.ul : R.ul;
  const float Kp = left ? L.p : R.p, Ke = left ? L.e : R.e, Ky = left ? L.y : R.y;
  const float SK = left ? SL : SR;
  // F_K + S_K (U*_K - U_K) is the physical flux of the star state U*_K
  // (star_region_euler.c:3-40): mass flux rho* S*, pressure
  // p* = p_K + rho_K (S_K - u_K)(S* - u_K), unchanged tangential velocity.
  // So one flux formula serves both cases, from the upwind state or its star
  // state, with one reciprocal.
  float m = Kmn, un = Kun, pp = Kp, ee = Ke;
  if (star) {
    const float dK = SK - Kun;
    const float inv = fast_rcp(SK - S_S);
    const float rdK = Kr * dK;
    const float cS = rdK * inv;  // rho*
    const float aK = S_S - Kun;
    m = cS * S_S;
    un = S_S;
    pp = fmaf(rdK, aK, Kp);
    // E* = rho* [E_K / rho_K + (S* - u_K)(S* + p_K / (rho_K (S_K - u_K)))]
    if (MODEL == 1) ee = fmaf(cS * aK, S_S, inv * fmaf(aK, Kp, dK * Ke));
  }
  const float F0 = m;
  const float Fa = fmaf(m, un, pp);
  const float Fb = m * Kum;
  const float Fc = m * Kul;
  const float F4 = MODEL == 1 ? (ee + pp) * un : m * Ky;
  Fn[0] = F0;
  frame_out<F>(f, Fa, Fb, Fc, Fn);
  Fn[4] = F4;
  return ok;
}

// Canonical flux of a face from the lower / upper face values (bc > 0: a
// domain-boundary face, the upper side is the ghost of the lower one).
template <int MODEL, int F = -1>
__device__ __forceinline__ bool canonical_flux(const MixedConst &mc, int f, int bc, bool clip,
                                               const float lo[kNeqMax], const float hi[kNeqMax],
                                               float Fn[kNeqMax]) {
  LS Ls, Rs;
  bool ok = local_state<MODEL, F>(mc, f, lo, clip, Ls);
  if (bc > 0) {
    Rs = Ls;
    local_ghost<MODEL, F>(mc, bc, f, Rs);
  } else {
    ok &= local_state<MODEL, F>(mc, f, hi, clip, Rs);
  }
  ok &= local_hllc<MODEL, F>(mc, f, bc, Ls, Rs, Fn);
  return ok;
}

// Minmod-limited slope of one variable towards a face (reconctruct_V3.c:17-43,
// slopes divided by dist_cc as multiplications) from the delta across the
// face (d0) and across the opposite face (d1): zero unless the face is active
// (not a domain boundary), |d0| > 1e-10 and sm * sp > 0; then the slope of
// smaller magnitude.  Selects rather than branches.  A NaN product (a domain
// boundary behind the cell has 1/dist_cc = inf and a zero delta) gives zero,
// as in the reference.
__device__ __forceinline__ float minmod_slope(bool active, float d0, float d1, float inv_p, float inv_m) {
  const float sp = d0 * inv_p, sm = -d1 * inv_m;
  const float m = fabsf(sm) > fabsf(sp) ? sp : sm;
  return (active && fabsf(d0) > 1e-10f && sm * sp > 0.0f) ? m : 0.0f;
}

// Minmod face value of face f of a cell with geometry code gx from its state
// and the deltas across f (d0) and across the opposite face (d1).
__device__ __forceinline__ void recon_face(const GeoTables *geo, int32_t gx, int f, const float qx[kNeqMax],
                                           const float d0[kNeqMax], const float d1[kNeqMax],
                                           float out[kNeqMax]) {
  const int lev = level_of(gx);
  const int rf = rel_of(gx, f), ro = rel_of(gx, opp_face(f));
  const float *gf = geo_face(geo, lev, f, rf);
  const float dcf = gf[0], inv_p = gf[1];
  const float inv_m = geo_face(geo, lev, opp_face(f), ro)[1];
#pragma unroll
  for (int v = 0; v < kNeqMax; ++v)
    out[v] = fmaf(dcf, minmod_slope(rf != kRelBoundary, d0[v], d1[v], inv_p, inv_m), qx[v]);
}

template <int NT = kBlock>  // threads of the block
__device__ __forceinline__ void block_max_lambda_f(float lam, double *out) {
  __shared__ float red[NT / 32];
  for (int o = 16; o > 0; o >>= 1) lam = fmaxf(lam, __shfl_xor_sync(0xffffffffu, lam, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = lam;
  __syncthreads();
  if (threadIdx.x == 0) {
    float mx = red[0];
    for (int w = 1; w < NT / 32; ++w) mx = fmaxf(mx, red[w]);
    const double d = double(mx);
    if (d > 0.0 || isnan(d)) atomicMax((unsigned long long *)out, (unsigned long long)__double_as_longlong(d));
  }
}

// CFL spectral radius of one cell (definition in fvgpu.h), FP32, with the
// area of face f from area(f) and 1 / (2 V).
template <int MODEL, class AreaFn>
__device__ __forceinline__ float cell_lambda_with(const MixedConst &mc, const float q[kNeqMax], AreaFn area,
                                                  float inv2vol) {
  FS s;
  mixed_face_state<MODEL>(mc, q, false, s);
  float acc = 0.0f;
#pragma unroll
  for (int f = 0; f < 6; ++f) {
    const float un = fabsf(fmaf(s.w, mc.fr[9 * f + 2], fmaf(s.v, mc.fr[9 * f + 1], s.u * mc.fr[9 * f])));
    acc = fmaf(area(f), un + s.c, acc);
  }
  return acc * inv2vol;
}

template <int MODEL>
__device__ __forceinline__ float cell_lambda_f(const MixedConst &mc, const GeoTables *geo, int32_t g,
                                               const float q[kNeqMax]) {
  const int lev = level_of(g);
  return cell_lambda_with<MODEL>(
      mc, q,
      [&](int f) {
        const int rel = rel_of(g, f);
        return rel == kRelFiner ? 4.0f * geo->sub_area[lev * 6 + f] : geo_face(geo, lev, f, rel)[2];
      },
      geo->inv2vol[lev]);
}

// RK stage update of one cell in increment form; FP64 state, FP32 copy and
// CFL radius at the last stage.  Returns the cell's CFL radius (0 otherwise).
template <int MODEL>
__device__ __forceinline__ bool stage_update(const MixedConst &mc, const StageArgs &a, int c, float dtv,
                                             const float R[kNeqMax], bool ok, float qn[kNvMax]) {
  const int n = a.n;
  bool finite = true;
#pragma unroll
  for (int v = 0; v < kNeqMax; ++v)
    if (!isfinite(R[v])) finite = false;
  if (!(ok && finite)) raise_error(a.err, ok ? kErrNonFinite : kErrRegion, c);
  // the stage-input increment, read again here rather than kept in
  // registers through the flux phase
  float din[kNeqMax] = {0.f, 0.f, 0.f, 0.f, 0.f};
  if (a.Din) {
#pragma unroll
    for (int v = 0; v < kNeqMax; ++v) din[v] = __ldg(a.Din + v * n + c);
  }
  // stage weight w: D_k = w (D_in + dt/V R), RK(1) D1 = dt/V R as such
  const float w = a.irk == 2 ? 0.25f : (a.irk == 3 ? (2.0f / 3.0f) : 0.5f);
  const bool first = a.irk == 1;
  float dn[kNeqMax];
#pragma unroll
  for (int v = 0; v < kNeqMax; ++v) {
    const float incr = dtv * R[v];
    dn[v] = first ? incr : w * (din[v] + incr);
  }
  if (a.last) {
    double snew[kNeqMax];
#pragma unroll
    for (int v = 0; v < kNeqMax; ++v) {
      snew[v] = __ldg(a.SN + v * n + c) + double(dn[v]);
      a.SNout[v * n + c] = snew[v];
    }
    to_state_words<MODEL>(snew, qn);
#pragma unroll
    for (int v = 0; v < kNv<MODEL>; ++v) a.SNfout[v * n + c] = qn[v];
    return true;
  }
#pragma unroll
  for (int v = 0; v < kNeqMax; ++v) {
    a.Dout[v * n + c] = dn[v];
    a.Sout[v * n + c] = __ldg(a.SNf + v * n + c) + dn[v];  // the value the next stage would form
  }
  if constexpr (MODEL == 3) {  // paired words: the next stage's input as a pair
#pragma unroll
    for (int v = 0; v < kNeqMax; v += 4) {
      float w[kNvMax];
      w[v] = __ldg(a.SNf + v * n + c);
      w[lo_word(v)] = __ldg(a.SNf + lo_word(v) * n + c);
      set_pair_ff(w, v, ff_add(pair_ff(w, v), FF{dn[v], 0.0f}));
      a.Sout[v * n + c] = w[v];
      a.Sout[lo_word(v) * n + c] = w[lo_word(v)];
    }
  }
  return false;
}

// stage state of any cell from global memory (SNf + D, written by the
// previous stage)
template <int MODEL>
__device__ __forceinline__ void global_state(const StageArgs &a, int x, float *q) {
#pragma unroll
  for (int v = 0; v < kNv<MODEL>; ++v) q[v] = __ldg(a.Sin + v * a.n + x);
}

// ============================ viscous terms =================================

// Cartesian velocity of the ghost across a boundary face f (bc.c:19-49) from
// the own face values q.
template <int MODEL>
__device__ __forceinline__ void ghost_velocity(const MixedConst &mc, int bc, int f, const float *q, float u[3]) {
  if (bc == 1) {  // the inflow state (state form: model 3 holds rho - kRhoOff)
    const float rinv = fast_rcp(MODEL == 3 ? mc.inflow[0] + kRhoOffF : mc.inflow[0]);
    u[0] = mc.inflow[1] * rinv;
    u[1] = mc.inflow[2] * rinv;
    u[2] = mc.inflow[3] * rinv;
    return;
  }
  const float rinv = fast_rcp(state_rho<MODEL>(q));
  u[0] = q[1] * rinv;
  u[1] = q[2] * rinv;
  u[2] = q[3] * rinv;
  if (bc == 3) {  // slip wall: normal component mirrored
    const float nx = mc.fr[9 * f], ny = mc.fr[9 * f + 1], nz = mc.fr[9 * f + 2];
    const float un = fmaf(u[2], nz, fmaf(u[1], ny, u[0] * nx));
    u[0] = fmaf(-2.0f * un, nx, u[0]);
    u[1] = fmaf(-2.0f * un, ny, u[1]);
    u[2] = fmaf(-2.0f * un, nz, u[2]);
  } else if (bc == 4) {  // no-slip wall: reversed
    u[0] = -u[0];
    u[1] = -u[1];
    u[2] = -u[2];
  }
}

// FV . n of one face (flux_viscous.c:57-232 with turb = 0) from the face
// values of both sides (bc > 0: a boundary face, the other side is the
// ghost of lo) and the momentum gradients of both cells, FP32.
template <int MODEL>
__device__ __forceinline__ void viscous_normal(const MixedConst &mc, int f, int bc, const float *lo, const float *hi,
                                               const float gl[9], const float gh[9], float FVn[kNeqMax]) {
  float ul[3], uh[3];
  {
    const float rinv = fast_rcp(state_rho<MODEL>(lo));
    ul[0] = lo[1] * rinv;
    ul[1] = lo[2] * rinv;
    ul[2] = lo[3] * rinv;
  }
  if (bc > 0) {
    ghost_velocity<MODEL>(mc, bc, f, lo, uh);
  } else {
    const float rinv = fast_rcp(state_rho<MODEL>(hi));
    uh[0] = hi[1] * rinv;
    uh[1] = hi[2] * rinv;
    uh[2] = hi[3] * rinv;
  }
  const float uf = 0.5f * (ul[0] + uh[0]), vf = 0.5f * (ul[1] + uh[1]), wf = 0.5f * (ul[2] + uh[2]);
  float g[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) g[i] = 0.5f * (gl[i] + gh[i]);
  const float mu = mc.visc;
  const float D = g[0] + g[4] + g[8];
  const float txx = mu * fmaf(2.0f, g[0], -(2.0f / 3.0f) * D);
  const float tyy = mu * fmaf(2.0f, g[4], -(2.0f / 3.0f) * D);
  const float tzz = mu * fmaf(2.0f, g[8], -(2.0f / 3.0f) * D);
  const float txy = mu * (g[1] + g[3]), txz = mu * (g[2] + g[6]), tyz = mu * (g[5] + g[7]);
  const float nx = mc.fr[9 * f], ny = mc.fr[9 * f + 1], nz = mc.fr[9 * f + 2];
  FVn[0] = 0.0f;
  FVn[1] = fmaf(txz, nz, fmaf(txy, ny, txx * nx));
  FVn[2] = fmaf(tyz, nz, fmaf(tyy, ny, txy * nx));
  FVn[3] = fmaf(tzz, nz, fmaf(tyz, ny, txz * nx));
  FVn[4] = 0.0f;
  if (mc.eos == 1) {
    const float ex = fmaf(wf, txz, fmaf(vf, txy, uf * txx));
    const float ey = fmaf(wf, tyz, fmaf(vf, tyy, uf * txy));
    const float ez = fmaf(wf, tzz, fmaf(vf, tyz, uf * txz));
    FVn[4] = fmaf(ez, nz, fmaf(ey, ny, ex * nx));
  }
}

__device__ __forceinline__ void load_grad9f(const float *__restrict__ SG, int n, int c, float g[9]) {
#pragma unroll
  for (int i = 0; i < 9; ++i) g[i] = __ldg(SG + i * n + c);
}

// Green-Gauss momentum gradients of the stage-input state (gradcalc.c:9-47,
// rows of rho u, rho v, rho w), FP32, one cell per thread.
template <int MODEL>
__global__ void __launch_bounds__(kBlock)
    k_mixed_grad(MixedConst mc, StageArgs a, float *__restrict__ SGout, const __grid_constant__ GeoTables geo_tab) {
  const GeoTables *geo = &geo_tab;
  const int c = blockIdx.x * kBlock + threadIdx.x;
  const int n = a.n;
  if (c >= n) return;
  float q[kNvMax];
  global_state<MODEL>(a, c, q);
  const int32_t g = __ldg(a.geom + c);
  const int lev = level_of(g);
  const float inv_vol = geo->inv_vol[lev];
  float gr[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  for (int f = 0; f < 6; ++f) {
    const int32_t code = __ldg(a.nbr + f * n + c);
    const float nx = mc.fr[9 * f], ny = mc.fr[9 * f + 1], nz = mc.fr[9 * f + 2];
    auto add = [&](const float m[3], float A) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float h = 0.5f * (m[k] + q[1 + k]) * A * inv_vol;
        gr[k * 3 + 0] = fmaf(h, nx, gr[k * 3 + 0]);
        gr[k * 3 + 1] = fmaf(h, ny, gr[k * 3 + 1]);
        gr[k * 3 + 2] = fmaf(h, nz, gr[k * 3 + 2]);
      }
    };
    if (is_boundary(code)) {
      const int bc = -1 - code;
      float m[3];
      if (bc == 1) {
        m[0] = mc.inflow[1];
        m[1] = mc.inflow[2];
        m[2] = mc.inflow[3];
      } else {
        float u[3];
        ghost_velocity<MODEL>(mc, bc, f, q, u);
        const float rho = state_rho<MODEL>(q);
        m[0] = rho * u[0];
        m[1] = rho * u[1];
        m[2] = rho * u[2];
        if (bc != 3 && bc != 4) {
          m[0] = q[1];
          m[1] = q[2];
          m[2] = q[3];
        }
      }
      add(m, geo_face(geo, lev, f, kRelBoundary)[2]);
    } else if (is_hanging(code)) {
      const int32_t *k = a.hang_nbr + 4 * hang_index(code);
      const float A = geo->sub_area[lev * 6 + f];
      for (int s = 0; s < 4; ++s) {
        const int ks = __ldg(k + s);
        const float m[3] = {__ldg(a.Sin + 1 * n + ks), __ldg(a.Sin + 2 * n + ks), __ldg(a.Sin + 3 * n + ks)};
        add(m, A);
      }
    } else {
      const float m[3] = {__ldg(a.Sin + 1 * n + code), __ldg(a.Sin + 2 * n + code), __ldg(a.Sin + 3 * n + code)};
      add(m, geo_face(geo, lev, f, rel_of(g, f))[2]);
    }
  }
#pragma unroll
  for (int i = 0; i < 9; ++i) SGout[i * n + c] = gr[i];
}

// ============================ general kernel ================================

// Model 3: the minmod slope of a paired word as a pair (reconctruct_V3.c:17-43,
// as minmod_slope).
__device__ __forceinline__ FF minmod_slope_ff(bool active, FF d0, FF d1, float inv_p, float inv_m) {
  const FF sp = ff_mul_f(d0, inv_p), sm = ff_mul_f(ff_neg(d1), inv_m);
  const FF m = ff_sub(ff_abs(sm), ff_abs(sp)).hi > 0.0f ? sp : sm;
  const bool same_sign = (sm.hi > 0.0f && sp.hi > 0.0f) || (sm.hi < 0.0f && sp.hi < 0.0f);
  return (active && fabsf(d0.hi) > 1e-10f && same_sign) ? m : FF{0.0f, 0.0f};
}

// Model 3: face value of face f of a cell with geometry code gx from its
// state words and the values across f (nbf) and across the opposite face
// (nbo): the momentum as recon_face does, the paired words as pairs.
__device__ __forceinline__ void recon_face_m3(const GeoTables *geo, int32_t gx, int f, const float *qx,
                                              const float *nbf, const float *nbo, float *out) {
  const int lev = level_of(gx);
  const int rf = rel_of(gx, f), ro = rel_of(gx, opp_face(f));
  const float *gf = geo_face(geo, lev, f, rf);
  const float dcf = gf[0], inv_p = gf[1];
  const float inv_m = geo_face(geo, lev, opp_face(f), ro)[1];
  const bool act = rf != kRelBoundary;
#pragma unroll
  for (int v = 1; v < 4; ++v)
    out[v] = fmaf(dcf, minmod_slope(act, nbf[v] - qx[v], nbo[v] - qx[v], inv_p, inv_m), qx[v]);
#pragma unroll
  for (int v = 0; v < kNeqMax; v += 4) {
    const FF q = pair_ff(qx, v);
    const FF sl = minmod_slope_ff(act, ff_sub(pair_ff(nbf, v), q), ff_sub(pair_ff(nbo, v), q), inv_p, inv_m);
    set_pair_ff(out, v, ff_add(q, ff_mul_f(sl, dcf)));
  }
}

template <int MODEL>
struct Block {
  static constexpr int NV = kNv<MODEL>;
  const StageArgs &a;
  const MixedConst &mc;
  const GeoTables *geo;  // the kernel's by-value copy (constant bank)
  int c0, cnt;
  const float (*st)[kBlock];
  __device__ Block(const StageArgs &a_, const MixedConst &mc_, const GeoTables *geo_, int c0_, int cnt_,
                   const float (*st_)[kBlock])
      : a(a_), mc(mc_), geo(geo_), c0(c0_), cnt(cnt_), st(st_) {}
  __device__ __forceinline__ bool in_block(int x) const { return unsigned(x - c0) < unsigned(cnt); }
  __device__ __forceinline__ void state(int x, float *q) const {
    if (in_block(x)) {
#pragma unroll
      for (int v = 0; v < NV; ++v) q[v] = st[v][x - c0];
      return;
    }
    global_state<MODEL>(a, x, q);
  }
  // value across face f of cell x (deltavalues.c): single neighbour, mean of
  // the four fine ones (model 3: the paired words summed as pairs), or the
  // boundary ghost
  __device__ __forceinline__ void across(int x, int f, const float *own, float *nb) const {
    across_code(__ldg(a.nbr + f * a.n + x), f, own, nb);
  }
  // the same with the neighbour code of face f already at hand
  __device__ __forceinline__ void across_code(int32_t code, int f, const float *own, float *nb) const {
    if (code >= 0) {
      state(code, nb);
    } else if (is_hanging(code)) {
      const int32_t *k = a.hang_nbr + 4 * hang_index(code);
      float acc[kNeqMax] = {0.f, 0.f, 0.f, 0.f, 0.f};
      FF acc2[2] = {{0.0f, 0.0f}, {0.0f, 0.0f}};
#pragma unroll 1
      for (int s = 0; s < 4; ++s) {
        float q[kNvMax];
        state(__ldg(k + s), q);
#pragma unroll
        for (int v = 0; v < kNeqMax; ++v) acc[v] += q[v];
        if constexpr (MODEL == 3) {
          acc2[0] = ff_add(acc2[0], pair_ff(q, 0));
          acc2[1] = ff_add(acc2[1], pair_ff(q, 4));
        }
      }
#pragma unroll
      for (int v = 0; v < kNeqMax; ++v) nb[v] = 0.25f * acc[v];
      if constexpr (MODEL == 3) {  // a quarter of a pair is exact
        set_pair_ff(nb, 0, FF{0.25f * acc2[0].hi, 0.25f * acc2[0].lo});
        set_pair_ff(nb, 4, FF{0.25f * acc2[1].hi, 0.25f * acc2[1].lo});
      }
    } else {
      boundary_value<MODEL>(mc, -1 - code, f, own, nb);
    }
  }
  // face value of face f of any cell (used across block edges)
  __device__ __forceinline__ void recon_any(int x, int f, float *out) const {
    float qx[kNvMax], nbp[kNvMax], nbm[kNvMax];
    state(x, qx);
    across(x, f, qx, nbp);
    across(x, opp_face(f), qx, nbm);
    if constexpr (MODEL == 3) {
      recon_face_m3(geo, __ldg(a.geom + x), f, qx, nbp, nbm, out);
    } else {
      float d0[kNeqMax], d1[kNeqMax];
#pragma unroll
      for (int v = 0; v < kNeqMax; ++v) {
        d0[v] = nbp[v] - qx[v];
        d1[v] = nbm[v] - qx[v];
      }
      recon_face(geo, __ldg(a.geom + x), f, qx, d0, d1, out);
    }
  }
};

// The flux(es) through one face of a cell of a general block, added to the
// cell's residual R (a 1:4 face: its four sub-faces in order).  P_ >= 0: a
// + face known at compile time; P_ < 0: face f_rt, a + face when plus_rt.
// A + face's flux is always computed, in the frame of that face, and
// published for the upper cell when the face has a single neighbour; a -
// face reads the published flux when the lower cell is in the block and its
// + face carries this cell alone, and otherwise recomputes the canonical
// flux (lower side first, frame of the lower cell's + face; a
// domain-boundary face in its own frame).
template <int MODEL, bool MUSCL>
struct FaceCtx {
  static constexpr int NV = kNv<MODEL>;
  const Block<MODEL> &blk;
  const MixedConst &mc;
  const StageArgs &a;
  const GeoTables *geo;
  int32_t g;
  int lev, t, c;
  float (*sf)[NV][kBlock];
  float (*fp)[kNeqMax][kBlock];

  template <int P_>
  __device__ __forceinline__ void face(int f_rt, bool plus_rt, int32_t code, float R[kNeqMax], bool &ok,
                                       const float *gown = nullptr) const {
    const bool plus = P_ >= 0 || plus_rt;
    const int f = P_ >= 0 ? P_ : f_rt;
    const int fo = opp_face(f);
    const int c0 = blk.c0;
    const bool boundary = is_boundary(code);
    const bool hanging = is_hanging(code);
    const int rel = rel_of(g, f);
    const int nsub = hanging ? 4 : 1;
    const int32_t *hk = hanging ? a.hang_nbr + 4 * hang_index(code) : nullptr;
    const float A = hanging ? geo->sub_area[lev * 6 + f] : geo_face(geo, lev, f, rel)[2];
#pragma unroll 1
    for (int s = 0; s < nsub; ++s) {
      const int other = boundary ? -1 : (hanging ? __ldg(hk + s) : code);
      float Fn[kNeqMax];
      const bool published = !plus && !boundary && (hanging || rel == kRelSame) && blk.in_block(other);
      if (published) {
        const int tl = other - c0;
#pragma unroll
        for (int v = 0; v < kNeqMax; ++v) Fn[v] = fp[plus_slot(fo)][v][tl];
      } else {
        float own[kNvMax], oth[kNvMax];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          own[v] = sf[f][v][t];
          oth[v] = own[v];
        }
        if (!boundary) {
          if (blk.in_block(other)) {
#pragma unroll
            for (int v = 0; v < NV; ++v) oth[v] = sf[fo][v][other - c0];
          } else if (MUSCL) {
            blk.recon_any(other, fo, oth);
          } else {
            blk.state(other, oth);
          }
        }
        const bool own_low = plus || boundary;
        float lo[kNvMax], hi[kNvMax];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          lo[v] = own_low ? own[v] : oth[v];
          hi[v] = own_low ? oth[v] : own[v];
        }
        const int bc = boundary ? -1 - code : 0;
        if constexpr (P_ >= 0)
          ok &= canonical_flux<MODEL, P_>(mc, P_, bc, MUSCL, lo, hi, Fn);
        else
          ok &= canonical_flux<MODEL>(mc, own_low ? f : fo, bc, MUSCL, lo, hi, Fn);
        if (mc.ns == 1) {  // (F - FV).n + FH
          float gl[9], gh[9], FVn[kNeqMax];
          const int clo = own_low ? c : other, chi = own_low ? (boundary ? c : other) : c;
          if (P_ >= 0 && gown) {  // a + face: the lower cell is this one, its gradients at hand
#pragma unroll
            for (int i = 0; i < 9; ++i) gl[i] = gown[i];
          } else {
            load_grad9f(a.SG, a.n, clo, gl);
          }
          load_grad9f(a.SG, a.n, chi, gh);
          viscous_normal<MODEL>(mc, own_low ? f : fo, bc, lo, hi, gl, gh, FVn);
#pragma unroll
          for (int v = 0; v < kNeqMax; ++v) Fn[v] -= FVn[v];
        }
        if (plus && !boundary && !hanging) {
#pragma unroll
          for (int v = 0; v < kNeqMax; ++v) fp[plus_slot(f)][v][t] = Fn[v];
        }
      }
      const float sA = (plus || boundary) ? -A : A;
#pragma unroll
      for (int v = 0; v < kNeqMax; ++v) R[v] = R[v] + sA * Fn[v];  // separate roundings: equal and opposite face fluxes cancel exactly
    }
  }
};

// register budgets: model 1 four blocks per SM (64 registers, as shared
// memory allows), model 3 three (80 registers without spills; its 64 KB of
// shared memory fits three blocks)
template <int MODEL, bool MUSCL>
__global__ void __launch_bounds__(kBlock, MODEL == 3 ? 3 : 4)
    k_mixed_general(MixedConst mc, StageArgs a, const __grid_constant__ GeoTables geo_tab) {
  constexpr int NV = kNv<MODEL>;
  __shared__ float st[NV][kBlock];
  __shared__ float sf[6][NV][kBlock];
  __shared__ float fp[3][kNeqMax][kBlock];
  __shared__ float s_dt;
  const BlockDesc bd = a.blocks[blockIdx.x];
  const int t = threadIdx.x;
  const int c0 = bd.start;
  const int c = c0 + t;
  const int n = a.n;
  const bool active = t < bd.count;
  constexpr bool muscl = MUSCL;
  const GeoTables *geo = &geo_tab;
  Block<MODEL> blk(a, mc, geo, c0, bd.count, st);

  // A: own stage state
  float q[kNvMax];
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    q[v] = active ? __ldg(a.Sin + v * n + c) : 0.0f;
    st[v][t] = q[v];
  }
  int32_t nb[6];
  int32_t g = 0;
#pragma unroll
  for (int f = 0; f < 6; ++f) nb[f] = active ? __ldg(a.nbr + f * n + c) : -3;
  if (active) g = __ldg(a.geom + c);
  if (t == 0) s_dt = __double2float_rn(*a.dt);
  __syncthreads();

  // B: own face values
  if (active) {
    if (muscl && MODEL == 3) {
      // one axis at a time: the values across its two faces, both face values
#pragma unroll 1
      for (int f = 0; f < 6; ++f) {
        if (f == 2 || f == 3 || f == 5) continue;  // the lower face of each pair carries the axis
        const int fo = opp_face(f);
        float nbf[kNvMax], nbo[kNvMax], o[kNvMax];
        blk.across_code(nb[f], f, q, nbf);
        blk.across_code(nb[fo], fo, q, nbo);
        recon_face_m3(geo, g, f, q, nbf, nbo, o);
#pragma unroll
        for (int v = 0; v < NV; ++v) sf[f][v][t] = o[v];
        recon_face_m3(geo, g, fo, q, nbo, nbf, o);
#pragma unroll
        for (int v = 0; v < NV; ++v) sf[fo][v][t] = o[v];
      }
    } else if (muscl) {
      float dl[6][kNeqMax];
#pragma unroll
      for (int f = 0; f < 6; ++f) {
        float nbv[kNeqMax];
        blk.across_code(nb[f], f, q, nbv);
#pragma unroll
        for (int v = 0; v < kNeqMax; ++v) dl[f][v] = nbv[v] - q[v];
      }
#pragma unroll
      for (int f = 0; f < 6; ++f) {
        float o[kNeqMax];
        recon_face(geo, g, f, q, dl[f], dl[opp_face(f)], o);
#pragma unroll
        for (int v = 0; v < kNeqMax; ++v) sf[f][v][t] = o[v];
      }
    } else {
#pragma unroll
      for (int f = 0; f < 6; ++f)
#pragma unroll
        for (int v = 0; v < NV; ++v) sf[f][v][t] = q[v];
    }
  }
  __syncthreads();

  // C: fluxes, + faces (publish), barrier, - faces.  Model 1 lays its +
  // faces out one by one with the face known at compile time (frames as
  // register choices, fixed shared-memory slots; measured faster on the
  // viscous Taylor-Green mesh) and shares one loop among the - faces, mostly
  // read from the published + fluxes; model 3, whose float-float flux code
  // is larger, runs all six faces through one loop (measured faster on the
  // bubble).
  float R[kNeqMax] = {0.f, 0.f, 0.f, 0.f, 0.f};
  bool ok = true;
  const int lev = level_of(g);
  const FaceCtx<MODEL, MUSCL> fc{blk, mc, a, geo, g, lev, t, c, sf, fp};
  if constexpr (MODEL == 1) {
    if (active) {
      float gown[9];
      if (mc.ns == 1) load_grad9f(a.SG, n, c, gown);
      fc.template face<1>(1, true, nb[1], R, ok, gown);
      fc.template face<2>(2, true, nb[2], R, ok, gown);
      fc.template face<5>(5, true, nb[5], R, ok, gown);
    }
    __syncthreads();
    if (active) {
#pragma unroll 1
      for (int it = 3; it < 6; ++it) {
        const int f = face_of_iter(it);
        fc.template face<-1>(f, false, f == 3 ? nb[3] : (f == 0 ? nb[0] : nb[4]), R, ok);
      }
    }
  } else {
#pragma unroll 1
    for (int it = 0; it < 6; ++it) {
      if (it == 3) __syncthreads();
      if (!active) continue;
      const int f = face_of_iter(it);
      // the neighbour code by selects: indexing nb by the loop's face would
      // put the array in local memory
      const int32_t code = f == 1 ? nb[1] : f == 2 ? nb[2] : f == 5 ? nb[5] : f == 3 ? nb[3] : f == 0 ? nb[0] : nb[4];
      fc.template face<-1>(f, it < 3, code, R, ok);
    }
  }

  float lam = 0.0f;
  if (active) {
    float qn[kNvMax];
    const float dtv = s_dt * geo->inv_vol[level_of(g)];
    if (stage_update<MODEL>(mc, a, c, dtv, R, ok, qn) && a.lambda) lam = cell_lambda_f<MODEL>(mc, geo, g, qn);
  }
  if (a.last && a.lambda) block_max_lambda_f(lam, a.lambda);
}

// 4-byte asynchronous global -> shared copy (cp.async.ca)
__device__ __forceinline__ void cp_async4(float *dst, const float *src) {
  const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src) : "memory");
}

// ============================= brick kernel =================================

__host__ __device__ constexpr int morton_local(int x, int y, int z) {
  return (x & 1) | ((y & 1) << 1) | ((z & 1) << 2) | (((x >> 1) & 1) << 3) | (((y >> 1) & 1) << 4) |
         (((z >> 1) & 1) << 5) | (((x >> 2) & 1) << 6) | (((y >> 2) & 1) << 7);
}
__host__ __device__ constexpr int morton_x(int t) { return (t & 1) | (((t >> 3) & 1) << 1) | (((t >> 6) & 1) << 2); }
__host__ __device__ constexpr int morton_y(int t) { return ((t >> 1) & 1) | (((t >> 4) & 1) << 1) | (((t >> 7) & 1) << 2); }
__host__ __device__ constexpr int morton_z(int t) { return ((t >> 2) & 1) | (((t >> 5) & 1) << 1); }

// Brick shapes: a Morton-aligned block of BX x BY x BZ same-level cells (one
// thread per cell) staged with a 2-deep face halo in a tile of
// (BX + 4) x (BY + 4) x (BZ + 4) cells whose z-plane stride is padded by PAD
// so that the 32 Morton-ordered lanes of a warp read 32 different banks.
//   Brick8  8x8x4 (256 cells): uniform regions;
//   Brick4  4x4x4 (64 cells): the smaller same-level blocks of AMR meshes.
template <int BX_, int BY_, int BZ_, int PAD_>
struct BrickShape {
  static constexpr int BX = BX_, BY = BY_, BZ = BZ_, N = BX_ * BY_ * BZ_;
  static constexpr int TX = BX + 4, TY = BY + 4, TZ = BZ + 4;
  static constexpr int P = TX * TY + PAD_;  // z-plane stride of the tile
  static constexpr int kTile = P * TZ;
  static constexpr int kFaces = (BX + 1) * BY * BZ + BX * (BY + 1) * BZ + BX * BY * (BZ + 1);
  static constexpr int kHalo = 2 * (2 * BY * BZ + 2 * BX * BZ + 2 * BX * BY);
  // flux slots: the +x, +y, +z faces of the N cells (axis * N + t), then
  // the faces on the brick's -x, -y, -z sides
  static constexpr int kSlotSideX = 3 * N, kSlotSideY = kSlotSideX + BY * BZ, kSlotSideZ = kSlotSideY + BX * BZ;
  // blocks per SM the launch bounds ask for: 48 registers at five 256-thread
  // blocks (measured faster than four), four for viscous runs (64 registers)
  static constexpr int kMinBlocks = 5 * 256 / N, kMinBlocksNS = 4 * 256 / N;
  __host__ __device__ static constexpr int tile_index(int x, int y, int z) {
    return (z + 2) * P + (y + 2) * TX + (x + 2);
  }
  __host__ __device__ static constexpr bool in_brick(int x, int y, int z) {
    return x >= 0 && x < BX && y >= 0 && y < BY && z >= 0 && z < BZ;
  }
  // bit f set when a brick cell lies on the brick's face-f side (0 for halo cells)
  __host__ __device__ static constexpr uint32_t edge_mask(int x, int y, int z) {
    if (!in_brick(x, y, z)) return 0u;
    return (y == 0 ? 1u : 0u) | (x == BX - 1 ? 2u : 0u) | (y == BY - 1 ? 4u : 0u) | (x == 0 ? 8u : 0u) |
           (z == 0 ? 16u : 0u) | (z == BZ - 1 ? 32u : 0u);
  }
  // faces on the brick's -z side: even rows y first, then odd ones, so that
  // a warp's lower cells fall in different banks of the tile
  __host__ __device__ static constexpr int zslot(int x, int y) {
    return (y & 1) * (BX * BY / 2) + (y >> 1) * BX + x;
  }
  __host__ __device__ static constexpr int zslot_y(int r) {
    return r < BX * BY / 2 ? 2 * (r / BX) : 2 * ((r - BX * BY / 2) / BX) + 1;
  }
  // a cell of the brick or of a neighbour brick (viscous runs read the
  // gradients of a face's two cells), 12 bits: a brick cell is its Morton
  // index; a cell of a neighbour brick has bit 11 set, the brick side in
  // bits 8-10 and its Morton index within that brick in bits 0-7
  __host__ __device__ static constexpr uint32_t cell_ref(int x, int y, int z) {
    if (in_brick(x, y, z)) return uint32_t(morton_local(x, y, z));
    const int side = x < 0 ? 3 : (x >= BX ? 1 : (y < 0 ? 0 : (y >= BY ? 2 : (z < 0 ? 4 : 5))));
    return 2048u | (uint32_t(side) << 8) | uint32_t(morton_local((x + BX) % BX, (y + BY) % BY, (z + BZ) % BZ));
  }
  static_assert(kTile <= 2048 && kFaces <= 1024 && kSlotSideZ + BX * BY == kFaces && N <= 256 && BY % 2 == 0,
                "brick table fields");
};
using Brick8 = BrickShape<8, 8, 4, 0>;
using Brick4 = BrickShape<4, 4, 4, 4>;

// Face tasks of a brick, in flux-slot order (Morton lanes of a warp then
// read tile cells in distinct shared-memory banks).  Packed: tile index of
// the lower cell (11 bits), axis (2), lower / upper cell inside the brick
// (1 + 1), edge masks of the lower and upper cells (6 + 6).
template <class S>
struct BrickTasks {
  uint32_t task[S::kFaces];
};
template <class S>
constexpr BrickTasks<S> make_brick_tasks() {
  BrickTasks<S> T{};
  for (int task = 0; task < S::kFaces; ++task) {
    int axis = 0, lx = 0, ly = 0, lz = 0;
    if (task < S::kSlotSideX) {
      axis = task / S::N;
      const int t = task % S::N;
      lx = morton_x(t);
      ly = morton_y(t);
      lz = morton_z(t);
    } else if (task < S::kSlotSideY) {
      const int r = task - S::kSlotSideX;
      lx = -1;
      ly = r % S::BY;
      lz = r / S::BY;
    } else if (task < S::kSlotSideZ) {
      const int r = task - S::kSlotSideY;
      axis = 1;
      lx = r % S::BX;
      ly = -1;
      lz = r / S::BX;
    } else {
      const int r = task - S::kSlotSideZ;
      axis = 2;
      lx = r % S::BX;
      ly = S::zslot_y(r);
      lz = -1;
    }
    const int ux = lx + (axis == 0), uy = ly + (axis == 1), uz = lz + (axis == 2);
    T.task[task] = uint32_t(S::tile_index(lx, ly, lz)) | (uint32_t(axis) << 11) |
                   (uint32_t(S::in_brick(lx, ly, lz)) << 13) | (uint32_t(S::in_brick(ux, uy, uz)) << 14) |
                   (S::edge_mask(lx, ly, lz) << 15) | (S::edge_mask(ux, uy, uz) << 21);
  }
  return T;
}
template <class S>
__device__ const BrickTasks<S> g_brick_tasks = make_brick_tasks<S>();

// The two cells of each face task (S::cell_ref), 12 bits each, lower first.
template <class S>
struct BrickTaskCells {
  uint32_t c[S::kFaces];
};
template <class S>
constexpr BrickTaskCells<S> make_brick_task_cells() {
  BrickTaskCells<S> C{};
  const BrickTasks<S> T = make_brick_tasks<S>();
  for (int task = 0; task < S::kFaces; ++task) {
    const uint32_t e = T.task[task];
    const int ti = int(e & 2047u), axis = int((e >> 11) & 3u);
    const int lz = ti / S::P - 2, rem = ti % S::P, ly = rem / S::TX - 2, lx = rem % S::TX - 2;
    C.c[task] = S::cell_ref(lx, ly, lz) | (S::cell_ref(lx + (axis == 0), ly + (axis == 1), lz + (axis == 2)) << 12);
  }
  return C;
}
template <class S>
__device__ const BrickTaskCells<S> g_brick_task_cells = make_brick_task_cells<S>();

// Halo cells of a brick, two layers beyond each side: the x sides, the y
// sides, the z sides.  Within each group the cells are dealt out round-robin
// over the tile's shared-memory banks, so that a warp's cells fall in as many
// different banks as the group has (all 32 for Brick8).  Packed: tile index
// (11 bits), brick side the cell lies beyond (3), Morton offset of the cell
// within its own brick (8).
template <class S>
struct BrickHalo {
  uint32_t h[S::kHalo];
};
template <class S>
constexpr BrickHalo<S> make_brick_halo() {
  BrickHalo<S> H{};
  int base = 0;
  for (int g = 0; g < 3; ++g) {
    const int na = g == 0 ? S::BY : S::BX, nb = g == 2 ? S::BY : S::BZ;  // extents of the in-plane axes
    const int ext = g == 0 ? S::BX : (g == 1 ? S::BY : S::BZ);           // extent along the group's axis
    const int count = 4 * na * nb;
    // bucket the group's cells by bank, then take one from every non-empty
    // bucket in turn
    uint32_t cell[4 * 8 * 8] = {};
    int bank_of[4 * 8 * 8] = {};
    int k = 0;
    for (int layer = 0; layer < 4; ++layer) {  // -2, -1, ext, ext + 1
      const int o = layer < 2 ? layer - 2 : ext + layer - 2;
      const int side = g == 0 ? (o < 0 ? 3 : 1) : (g == 1 ? (o < 0 ? 0 : 2) : (o < 0 ? 4 : 5));
      const int lo = o < 0 ? o + ext : o - ext;  // coordinate within the neighbour brick
      for (int b = 0; b < nb; ++b)
        for (int a2 = 0; a2 < na; ++a2) {
          int hx = a2, hy = b, hz = 0, lx = a2, ly = b, lz = 0;
          if (g == 0) {
            hx = o; lx = lo; hy = ly = a2; hz = lz = b;
          } else if (g == 1) {
            hy = o; ly = lo; hx = lx = a2; hz = lz = b;
          } else {
            hz = o; lz = lo; hx = lx = a2; hy = ly = b;
          }
          const int ti = S::tile_index(hx, hy, hz);
          cell[k] = uint32_t(ti) | (uint32_t(side) << 11) | (uint32_t(morton_local(lx, ly, lz)) << 14);
          bank_of[k] = ti % 32;
          ++k;
        }
    }
    int first[33] = {}, cursor[32] = {}, order[4 * 8 * 8] = {};
    for (int i = 0; i < count; ++i) ++first[bank_of[i] + 1];
    for (int bank = 0; bank < 32; ++bank) first[bank + 1] += first[bank];
    for (int bank = 0; bank < 32; ++bank) cursor[bank] = first[bank];
    for (int i = 0; i < count; ++i) order[cursor[bank_of[i]]++] = i;  // stable by bank
    for (int bank = 0; bank < 32; ++bank) cursor[bank] = first[bank];
    int out = 0;
    while (out < count)
      for (int bank = 0; bank < 32; ++bank)
        if (cursor[bank] < first[bank + 1]) H.h[base + out++] = cell[order[cursor[bank]++]];
    base += count;
  }
  return H;
}
template <class S>
__device__ const BrickHalo<S> g_brick_halo = make_brick_halo<S>();

// Brick cells in Morton order.  Word 0: tile index (11 bits), edge mask (6);
// word 1: flux slots of the cell's -x, -y, -z faces (10 bits each).  The +x,
// +y, +z faces are slots t, N + t, 2N + t.
template <class S>
struct BrickCells {
  uint32_t w[2 * S::N];
};
template <class S>
constexpr BrickCells<S> make_brick_cells() {
  BrickCells<S> C{};
  for (int t = 0; t < S::N; ++t) {
    const int x = morton_x(t), y = morton_y(t), z = morton_z(t);
    const int mx = x > 0 ? morton_local(x - 1, y, z) : S::kSlotSideX + y + S::BY * z;
    const int my = y > 0 ? S::N + morton_local(x, y - 1, z) : S::kSlotSideY + x + S::BX * z;
    const int mz = z > 0 ? 2 * S::N + morton_local(x, y, z - 1) : S::kSlotSideZ + S::zslot(x, y);
    C.w[2 * t] = uint32_t(S::tile_index(x, y, z)) | (S::edge_mask(x, y, z) << 11);
    C.w[2 * t + 1] = uint32_t(mx) | (uint32_t(my) << 10) | (uint32_t(mz) << 20);
  }
  return C;
}
template <class S>
__device__ const BrickCells<S> g_brick_cells = make_brick_cells<S>();

// CFL radius of a brick cell: the frames are axis-aligned (checked at
// upload), so |u.n| on face f is the magnitude of one velocity component --
// the same value cell_lambda_with forms from the frame, without it.
template <int MODEL>
__device__ __forceinline__ float brick_lambda(const MixedConst &mc, const float q[kNeqMax], uint32_t be,
                                              const float (*geo)[2][4], float inv2vol) {
  FS s;
  mixed_face_state<MODEL>(mc, q, false, s);
  const float au = fabsf(s.u), av = fabsf(s.v), aw = fabsf(s.w);
  float acc = 0.0f;
#pragma unroll
  for (int f = 0; f < 6; ++f) {
    const float un = (f == 1 || f == 3) ? au : ((f == 0 || f == 2) ? av : aw);
    acc = fmaf(geo[f][(be >> f) & 1u][2], un + s.c, acc);
  }
  return acc * inv2vol;
}

template <int MODEL, bool MUSCL, bool NS, class S>
__global__ void __launch_bounds__(S::N, NS ? S::kMinBlocksNS : S::kMinBlocks)
    k_mixed_brick(MixedConst mc, StageArgs a) {
  constexpr int BX = S::BX, BY = S::BY, BZ = S::BZ, TX = S::TX, NB = S::N;
  constexpr int kTile = S::kTile, kFaces = S::kFaces, kHalo = S::kHalo;
  constexpr int kSlotSideY = S::kSlotSideY, kSlotSideZ = S::kSlotSideZ;
  __shared__ float tile[kNeqMax][kTile];
  __shared__ float flux[kNeqMax][kFaces];
  __shared__ float s_geo[6][2][4];  // per face index, relation same / boundary: dcf, 1/dcc, area
  __shared__ float s_dtv, s_inv2vol;  // dt / V and 1 / (2 V) of the brick's level
  __shared__ int s_side[6];  // brick sides (indexed at run time: kept out of local memory)
  const BlockDesc *bdp = a.blocks + blockIdx.x;
  const int t = threadIdx.x;
  const int n = a.n;
  constexpr bool muscl = MUSCL;
  const int start = __ldg(&bdp->start), level = __ldg(&bdp->level);
  const int c = start + t;
  uint32_t bmask = 0;  // sides of the brick on the domain boundary
#pragma unroll
  for (int f = 0; f < 6; ++f)
    if (__ldg(&bdp->side[f]) < 0) bmask |= 1u << f;
  if (t < 6) s_side[t] = __ldg(&bdp->side[t]);
  if (t < 12) {
    const int f = t >> 1, r = t & 1;
    const float *gf = geo_face(a.geo, level, f, r ? kRelBoundary : kRelSame);
    s_geo[f][r][0] = gf[0];
    s_geo[f][r][1] = gf[1];
    s_geo[f][r][2] = gf[2];
  }
  if (t == 0) {
    s_dtv = __double2float_rn(*a.dt) * a.geo->inv_vol[level];
    s_inv2vol = a.geo->inv2vol[level];
  }

  // the arrays the update reads at the end, on their way to L2 (128-byte
  // lines: NB / 16 per FP64 variable, NB / 32 per FP32 one)
  constexpr int kL64 = NB / 16, kL32 = NB / 32;
  if (a.last && t < kNeqMax * kL64) {  // the FP64 step-start state
    const int v = t / kL64, l = t % kL64;
    asm volatile("prefetch.global.L2 [%0];" ::"l"(a.SN + int64_t(v) * n + start + 16 * l));
  }
  if (a.Din && t >= kNeqMax * kL64 && t < kNeqMax * (kL64 + kL32)) {  // the stage-input increment
    const int r = t - kNeqMax * kL64, v = r / kL32, l = r % kL32;
    asm volatile("prefetch.global.L2 [%0];" ::"l"(a.Din + int64_t(v) * n + start + 32 * l));
  }
  if (a.Din && !a.last && t >= kNeqMax * (kL64 + kL32) && t < kNeqMax * (kL64 + 2 * kL32)) {  // FP32 SN
    const int r = t - kNeqMax * (kL64 + kL32), v = r / kL32, l = r % kL32;
    asm volatile("prefetch.global.L2 [%0];" ::"l"(a.SNf + int64_t(v) * n + start + 32 * l));
  }
  static_assert(kNeqMax * (kL64 + 2 * kL32) <= NB, "prefetch lanes");
  // A1: the brick's cells and the halo from the six neighbour bricks, copied
  // global -> shared asynchronously (cp.async, no register round trip)
  {
    const int ti = int(__ldg(&g_brick_cells<S>.w[2 * t]) & 2047u);
#pragma unroll
    for (int v = 0; v < kNeqMax; ++v) cp_async4(&tile[v][ti], a.Sin + v * n + c);
  }
#pragma unroll
  for (int h = t; h < kHalo; h += NB) {
    const uint32_t e = __ldg(&g_brick_halo<S>.h[h]);
    const int base = __ldg(&bdp->side[(e >> 11) & 7u]);
    if (base >= 0) {
      const int ti = int(e & 2047u), x = base + int(e >> 14);
#pragma unroll
      for (int v = 0; v < kNeqMax; ++v) cp_async4(&tile[v][ti], a.Sin + v * n + x);
    }
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
  __syncthreads();
  // A2: ghost values beyond domain-boundary sides (deltavalues.c:9-14): the
  // ghost of the brick cell next to it, in both halo layers
  if (bmask) {
#pragma unroll 1
    for (int h = t; h < 2 * (BY * BZ + BX * BZ + BX * BY); h += NB) {
      int side, bx, by, bz, sx = 0, sy = 0, sz = 0;
      if (h < 2 * BY * BZ) {
        side = h < BY * BZ ? 3 : 1;
        const int rr = h % (BY * BZ);
        by = rr % BY;
        bz = rr / BY;
        bx = side == 3 ? 0 : BX - 1;
        sx = side == 3 ? -1 : 1;
      } else if (h < 2 * BY * BZ + 2 * BX * BZ) {
        const int hh = h - 2 * BY * BZ;
        side = hh < BX * BZ ? 0 : 2;
        const int rr = hh % (BX * BZ);
        bx = rr % BX;
        bz = rr / BX;
        by = side == 0 ? 0 : BY - 1;
        sy = side == 0 ? -1 : 1;
      } else {
        const int hh = h - 2 * BY * BZ - 2 * BX * BZ;
        side = hh < BX * BY ? 4 : 5;
        const int rr = hh % (BX * BY);
        bx = rr % BX;
        by = rr / BX;
        bz = side == 4 ? 0 : BZ - 1;
        sz = side == 4 ? -1 : 1;
      }
      if ((bmask >> side) & 1u) {
        float own[kNeqMax], gv[kNeqMax];
        const int ti_own = S::tile_index(bx, by, bz);
#pragma unroll
        for (int v = 0; v < kNeqMax; ++v) own[v] = tile[v][ti_own];
        boundary_value<MODEL>(mc, -1 - s_side[side], side, own, gv);
        const int t1 = S::tile_index(bx + sx, by + sy, bz + sz), t2 = S::tile_index(bx + 2 * sx, by + 2 * sy, bz + 2 * sz);
#pragma unroll
        for (int v = 0; v < kNeqMax; ++v) {
          tile[v][t1] = gv[v];
          tile[v][t2] = gv[v];
        }
      }
    }
    __syncthreads();  // bmask is uniform across the block
  }

  // face value of the face g of the tile cell at ti (edge mask e), with the
  // values across g at ti + dg and across the opposite face at ti - dg.
  // EDGE: the brick has a side on the domain boundary.
  auto recon_tile = [&](auto edge, int ti, uint32_t e, int g, int dg, float out[kNeqMax]) {
    constexpr bool EDGE = decltype(edge)::value;
    float qp[kNeqMax];
#pragma unroll
    for (int v = 0; v < kNeqMax; ++v) qp[v] = tile[v][ti];
    if (!muscl) {
#pragma unroll
      for (int v = 0; v < kNeqMax; ++v) out[v] = qp[v];
      return;
    }
    int rg = 0, ro = 0;
    if (EDGE) {
      const uint32_t be = e & bmask;
      rg = (be >> g) & 1u;
      ro = (be >> opp_face(g)) & 1u;
    }
    const float dcf = s_geo[g][rg][0], inv_p = s_geo[g][rg][1], inv_m = s_geo[opp_face(g)][ro][1];
#pragma unroll
    for (int v = 0; v < kNeqMax; ++v) {
      const float d0 = tile[v][ti + dg] - qp[v];
      const float d1 = tile[v][ti - dg] - qp[v];
      out[v] = fmaf(dcf, minmod_slope(!rg, d0, d1, inv_p, inv_m), qp[v]);
    }
  };

  // B: face tasks -- each face of the brick once
  // viscous runs: the global index of a face task's cell (S::cell_ref)
  // and the viscous normal flux of a face, subtracted as the general kernel
  // does: (F - FV).n + FH
  auto cell_of = [&](uint32_t r) -> int {
    return (r & 2048u) ? s_side[(r >> 8) & 7u] + int(r & 255u) : start + int(r & 255u);
  };
  auto sub_viscous = [&](int f, int bc, int clo, int chi, const float lo[kNeqMax], const float hi[kNeqMax],
                         float Fn[kNeqMax]) {
    float gl[9], gh[9], FVn[kNeqMax];
    load_grad9f(a.SG, n, clo, gl);
    load_grad9f(a.SG, n, chi, gh);
    viscous_normal<MODEL>(mc, f, bc, lo, hi, gl, gh, FVn);
#pragma unroll
    for (int v = 0; v < kNeqMax; ++v) Fn[v] -= FVn[v];
  };
  auto face_tasks = [&](auto edge) {
    constexpr bool EDGE = decltype(edge)::value;
    bool fok = true;
#pragma unroll 1
    for (int task = t; task < kFaces; task += NB) {
      const uint32_t e = __ldg(&g_brick_tasks<S>.task[task]);
      const int ti = int(e & 2047u);
      const int axis = int((e >> 11) & 3u);
      const bool low_in = (e >> 13) & 1u, up_in = (e >> 14) & 1u;
      const uint32_t elo = (e >> 15) & 63u, eup = (e >> 21) & 63u;
      const int st = axis == 0 ? 1 : (axis == 1 ? TX : S::P);
      const int fp = axis == 0 ? 1 : (axis == 1 ? 2 : 5);
      const int fm = opp_face(fp);
      float Fn[kNeqMax];
      const int bside = low_in ? fp : fm;
      if (EDGE && !(low_in && up_in) && s_side[bside] < 0) {
        // the brick cell's own domain-boundary face, own frame (residual_faces_AMR.c:196-209)
        float own[kNeqMax];
        if (low_in)
          recon_tile(edge, ti, elo, fp, st, own);
        else
          recon_tile(edge, ti + st, eup, fm, -st, own);
        fok &= canonical_flux<MODEL>(mc, bside, -1 - s_side[bside], muscl, own, own, Fn);
        if (NS) {
          const uint32_t cr = __ldg(&g_brick_task_cells<S>.c[task]);
          const int cown = cell_of(low_in ? (cr & 4095u) : (cr >> 12));
          sub_viscous(bside, -1 - s_side[bside], cown, cown, own, own, Fn);
        }
        if (!low_in) {  // stored as the +-face flux of the lower cell that is not there
#pragma unroll
          for (int v = 0; v < kNeqMax; ++v) Fn[v] = -Fn[v];
        }
      } else {
        float lo[kNeqMax], hi[kNeqMax];
        recon_tile(edge, ti, elo, fp, st, lo);
        recon_tile(edge, ti + st, eup, fm, -st, hi);
        fok &= canonical_flux<MODEL>(mc, fp, 0, muscl, lo, hi, Fn);
        if (NS) {
          const uint32_t cr = __ldg(&g_brick_task_cells<S>.c[task]);
          sub_viscous(fp, 0, cell_of(cr & 4095u), cell_of(cr >> 12), lo, hi, Fn);
        }
      }
#pragma unroll
      for (int v = 0; v < kNeqMax; ++v) flux[v][task] = Fn[v];
    }
    return fok;
  };
  // The same for a brick off the domain boundary: each thread its cell's +x,
  // +y, +z faces (slots t, N + t, 2N + t), then the first threads the faces on
  // the brick's lower sides; face index, stride and frame as compile-time
  // constants (the axis is uniform across each warp of an 8x8x4 brick).
  float R[kNeqMax] = {0.f, 0.f, 0.f, 0.f, 0.f};
  auto face_tasks_inner = [&]() {
    bool fok = true;
    const int ti_own = int(__ldg(&g_brick_cells<S>.w[2 * t]) & 2047u);
    auto inner = [&](auto fpc, int ti, int slot, bool own) {
      constexpr int FP = decltype(fpc)::value;
      constexpr int ST = FP == 1 ? 1 : (FP == 2 ? TX : S::P);
      float lo[kNeqMax], hi[kNeqMax], Fn[kNeqMax];
      recon_tile(std::false_type{}, ti, 0u, FP, ST, lo);
      recon_tile(std::false_type{}, ti + ST, 0u, opp_face(FP), -ST, hi);
      fok &= canonical_flux<MODEL, FP>(mc, FP, 0, muscl, lo, hi, Fn);
      if (NS) {
        const uint32_t cr = __ldg(&g_brick_task_cells<S>.c[slot]);
        sub_viscous(FP, 0, cell_of(cr & 4095u), cell_of(cr >> 12), lo, hi, Fn);
      }
#pragma unroll
      for (int v = 0; v < kNeqMax; ++v) flux[v][slot] = Fn[v];
      if (own) {  // the cell's own + face: its first residual terms, in order
        const float sA = -s_geo[FP][0][2];
#pragma unroll
        for (int v = 0; v < kNeqMax; ++v) R[v] = R[v] + sA * Fn[v];
      }
    };
    inner(std::integral_constant<int, 1>{}, ti_own, t, true);
    inner(std::integral_constant<int, 2>{}, ti_own, NB + t, true);
    inner(std::integral_constant<int, 5>{}, ti_own, 2 * NB + t, true);
    const int slot = 3 * NB + t;
    if (slot < kFaces) {
      const int ti = int(__ldg(&g_brick_tasks<S>.task[slot]) & 2047u);
      if (slot < kSlotSideY)
        inner(std::integral_constant<int, 1>{}, ti, slot, false);
      else if (slot < kSlotSideZ)
        inner(std::integral_constant<int, 2>{}, ti, slot, false);
      else
        inner(std::integral_constant<int, 5>{}, ti, slot, false);
    }
    return fok;
  };
  const bool ok = bmask ? face_tasks(std::true_type{}) : face_tasks_inner();
  __syncthreads();

  // C: gather in the fixed face order, RK stage update
  const uint32_t cw0 = __ldg(&g_brick_cells<S>.w[2 * t]), cw1 = __ldg(&g_brick_cells<S>.w[2 * t + 1]);
  const uint32_t be = (cw0 >> 11) & 63u & bmask;
  const int sx_m = int(cw1 & 1023u), sy_m = int((cw1 >> 10) & 1023u), sz_m = int(cw1 >> 20);
  // order +x, +y, +z, -x, -y, -z as in the general kernel
  auto add_face = [&](int f, int task, bool plus) {
    const float A = s_geo[f][(be >> f) & 1u][2];
    const float sA = plus ? -A : A;
#pragma unroll
    for (int v = 0; v < kNeqMax; ++v) R[v] = R[v] + sA * flux[v][task];  // as the general kernel
  };
  if (bmask) {  // a brick off the domain boundary added its + faces already
    add_face(1, t, true);
    add_face(2, NB + t, true);
    add_face(5, 2 * NB + t, true);
  }
  add_face(3, sx_m, false);
  add_face(0, sy_m, false);
  add_face(4, sz_m, false);
  float qn[kNvMax], lam = 0.0f;
  if (stage_update<MODEL>(mc, a, c, s_dtv, R, ok, qn) && a.lambda)
    lam = brick_lambda<MODEL>(mc, qn, be, s_geo, s_inv2vol);
  if (a.last && a.lambda) block_max_lambda_f<NB>(lam, a.lambda);
}

// FP32 copy of an FP64 state (after an upload or an FP64-path step), model
// 1: the count = neq * n values word for word.
__global__ void k_state_to_f32(const double *__restrict__ S, float *__restrict__ Sf, int64_t count) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += int64_t(gridDim.x) * blockDim.x)
    Sf[i] = __double2float_rn(S[i]);
}

// The same for model 3, one cell per thread: seven state words per cell.
__global__ void k_state_to_f32_m3(const double *__restrict__ S, float *__restrict__ Sf, int64_t n) {
  for (int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; c < n; c += int64_t(gridDim.x) * blockDim.x) {
    double x[kNeqMax];
    float q[kNvMax];
#pragma unroll
    for (int v = 0; v < kNeqMax; ++v) x[v] = S[v * n + c];
    to_state_words<3>(x, q);
#pragma unroll
    for (int v = 0; v < kNv<3>; ++v) Sf[v * n + c] = q[v];
  }
}

// The same with the CFL spectral radius of the copied state (the mixed
// path's first CFL time step after an upload): one cell per thread.
template <int MODEL>
__global__ void __launch_bounds__(kBlock) k_state_to_f32_lambda(MixedConst mc, const int32_t *__restrict__ geom,
                                                                const GeoTables *geo, const double *__restrict__ S,
                                                                float *__restrict__ Sf, int n, double *lambda) {
  float lam = 0.0f;
  for (int c = blockIdx.x * kBlock + threadIdx.x; c < n; c += gridDim.x * kBlock) {
    double x[kNeqMax];
    float q[kNvMax];
#pragma unroll
    for (int v = 0; v < kNeqMax; ++v) x[v] = S[int64_t(v) * n + c];
    to_state_words<MODEL>(x, q);
#pragma unroll
    for (int v = 0; v < kNv<MODEL>; ++v) Sf[int64_t(v) * n + c] = q[v];
    lam = fmaxf(lam, cell_lambda_f<MODEL>(mc, geo, __ldg(geom + c), q));
  }
  block_max_lambda_f(lam, lambda);
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
  // the inflow ghost in FP32 state form (model 3: the paired words of
  // rho - kRhoOff and rho Y; the library accepts inflow boundaries for model
  // 1 only)
  for (int v = 0; v < kNeqMax; ++v) mc.inflow[v] = float(ph.inflow[v]);
  if (ph.model == 3) {
    for (int v = 0; v < kNeqMax; v += 4) {
      const double x = v == 0 ? ph.inflow[0] - kRhoOffD : ph.inflow[4];
      mc.inflow[v] = float(x);
      mc.inflow[lo_word(v)] = float(x - double(mc.inflow[v]));
    }
  }
  mc.model = ph.model;
  mc.neq = ph.neq;
  mc.ischeme = ph.ischeme;
  mc.visc = float(ph.visc);
  mc.ns = ph.ns;
  mc.eos = ph.eos;
  return mc;
}

// resource slots
enum {
  kBufGeom = 0, kBufTables = 1, kBufD1 = 2, kBufD2 = 3, kBufAlt = 4, kBufSNf = 5, kBufSNfAlt = 6, kBufBlocks = 7,
  kBufX1 = 8, kBufX2 = 9, kBufSG = 10
};

cudaError_t alloc_slot(MixedResources &r, int slot, size_t bytes) {
  const size_t want = bytes ? bytes : 16;
  if (r.buf[slot] && want <= r.cap[slot]) {  // an earlier mesh's buffer is large enough
    r.bytes[slot] = bytes;
    return cudaSuccess;
  }
  if (r.buf[slot]) cudaFree(r.buf[slot]);
  r.buf[slot] = nullptr;
  r.bytes[slot] = 0;
  r.cap[slot] = 0;
  cudaError_t e = cudaMalloc(&r.buf[slot], want);
  if (e == cudaSuccess) {
    r.bytes[slot] = bytes;
    r.cap[slot] = want;
  }
  return e;
}

StageArgs stage_args(MixedResources &r, const MeshView &m) {
  StageArgs a{};
  a.n = int(m.n);
  a.nbr = m.nbr;
  a.geom = static_cast<const int32_t *>(r.buf[kBufGeom]);
  a.hang_nbr = m.hang_nbr;
  a.geo = static_cast<const GeoTables *>(r.buf[kBufTables]);
  return a;
}

// ---- host: brick detection ---------------------------------------------------

int host_morton_local(int x, int y, int z) {
  return (x & 1) | ((y & 1) << 1) | ((z & 1) << 2) | (((x >> 1) & 1) << 3) | (((y >> 1) & 1) << 4) |
         (((z >> 1) & 1) << 5) | (((x >> 2) & 1) << 6) | (((y >> 2) & 1) << 7);
}
void host_morton_decode(int t, int &x, int &y, int &z) {
  x = (t & 1) | (((t >> 3) & 1) << 1) | (((t >> 6) & 1) << 2);
  y = ((t >> 1) & 1) | (((t >> 4) & 1) << 1) | (((t >> 7) & 1) << 2);
  z = ((t >> 2) & 1) | (((t >> 5) & 1) << 1);
}
constexpr int kStepX[6] = {0, 1, 0, -1, 0, 0}, kStepY[6] = {-1, 0, 1, 0, 0, 0}, kStepZ[6] = {0, 0, 0, 0, -1, 1};

// cells i..i+N-1 form a BX x BY x BZ same-level block in local Morton order
// whose internal face links are the block's own
template <class S>
bool brick_interior(const fvgpu_mesh_soa *m, int64_t i) {
  const int64_t n = m->ncells;
  if (i + S::N > n) return false;
  const int lev = m->level[i];
  // quick rejects: the corner cell's +x/+y/+z neighbours
  if (m->nbr[1 * n + i] != i + 1 || m->nbr[2 * n + i] != i + 2 || m->nbr[5 * n + i] != i + 4) return false;
  for (int t = 0; t < S::N; ++t) {
    if (m->level[i + t] != lev) return false;
    int x, y, z;
    host_morton_decode(t, x, y, z);
    for (int f = 0; f < 6; ++f) {
      const int nx = x + kStepX[f], ny = y + kStepY[f], nz = z + kStepZ[f];
      if (!S::in_brick(nx, ny, nz)) continue;
      if (m->nbr[int64_t(f) * n + i + t] != i + host_morton_local(nx, ny, nz)) return false;
    }
  }
  return true;
}

// the starts of all same-level Morton blocks of shape S
template <class S>
void find_blocks(const fvgpu_mesh_soa *m, std::vector<char> &is_block) {
  const int64_t n = m->ncells;
  for (int64_t i = 0; i + S::N <= n;) {
    if (brick_interior<S>(m, i)) {
      is_block[size_t(i)] = 1;
      i += S::N;
    } else {
      ++i;
    }
  }
}

// side f of brick i: the first cell of a same-level Morton block of the same
// shape that supplies all its neighbours, -1-bc for a uniform domain
// boundary, or INT_MIN
template <class S>
int brick_side(const fvgpu_mesh_soa *m, int64_t i, int f, const std::vector<char> &is_block) {
  const int64_t n = m->ncells;
  int result = 0;
  bool first = true;
  for (int t = 0; t < S::N; ++t) {
    int x, y, z;
    host_morton_decode(t, x, y, z);
    const int nx = x + kStepX[f], ny = y + kStepY[f], nz = z + kStepZ[f];
    if (S::in_brick(nx, ny, nz)) continue;  // interior face
    const int32_t code = m->nbr[int64_t(f) * n + i + t];
    int value;
    if (code < 0 && code > FVGPU_HANG0) {
      value = code;  // boundary -1 - bc
    } else if (code >= 0) {
      const int wx = (nx + S::BX) % S::BX, wy = (ny + S::BY) % S::BY, wz = (nz + S::BZ) % S::BZ;
      const int64_t base = int64_t(code) - host_morton_local(wx, wy, wz);
      if (base < 0 || base + S::N > n || !is_block[size_t(base)]) return INT32_MIN;
      if (m->level[code] != m->level[i]) return INT32_MIN;
      value = int(base);
    } else {
      return INT32_MIN;  // 1:4 face
    }
    if (first) {
      result = value;
      first = false;
    } else if (value != result) {
      return INT32_MIN;
    }
  }
  return result;
}

template <class S>
bool brick_sides_resolve(const fvgpu_mesh_soa *m, int64_t i, const std::vector<char> &is_block) {
  for (int f = 0; f < 6; ++f)
    if (brick_side<S>(m, i, f, is_block) == INT32_MIN) return false;
  return true;
}

// Geometry of two faces is the same for the FP32 tables when the FP32 values
// agree to a few ulps: the FP64 areas and distances follow the reference's
// node-coordinate arithmetic and vary in the last bits from cell to cell
// where the box length is not a power of two.
static bool same_geo(float a, float b) {
  if (a == b) return true;
  const float m = fabsf(a) > fabsf(b) ? fabsf(a) : fabsf(b);
  return fabsf(a - b) <= 4e-7f * m;
}

}  // namespace

int mixed_prepare_host(MixedResources &r, const Phys &ph, const fvgpu_mesh_soa *m, char *why, size_t whylen) {
  r.ready = false;
  r.snf_valid = false;
  char tmp[256];
  if (!mixed_supported(ph, tmp, sizeof tmp)) {
    snprintf(why, whylen, "%s", tmp);
    return FVGPU_ERR_UNSUPPORTED;
  }
  if (!m->level) {
    snprintf(why, whylen, "the mixed path needs the per-cell level array");
    return FVGPU_ERR_UNSUPPORTED;
  }
  // fluxes are evaluated in the face frames of the reference's hexahedral
  // cells, compiled in as signed permutations
  for (int f = 0; f < 6; ++f)
    for (int k = 0; k < 9; ++k)
      if (m->frames[9 * f + k] != double(std_frame(f, k))) {
        snprintf(why, whylen, "the mixed path needs the hexahedral cells' face frames (face %d)", f);
        return FVGPU_ERR_UNSUPPORTED;
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
          if (!same_geo(float(m->hang_area[4 * h + s]), sa)) {
            snprintf(why, whylen, "the mixed path needs equal sub-face areas");
            return FVGPU_ERR_UNSUPPORTED;
          }
        const int k = lev * 6 + f;
        if (!seen_sub[k]) {
          seen_sub[k] = 1;
          gt.sub_area[k] = sa;
        } else if (!same_geo(gt.sub_area[k], sa)) {
          snprintf(why, whylen, "the mixed path needs one sub-face area per level and face");
          return FVGPU_ERR_UNSUPPORTED;
        }
        if (m->nbr_face[i] != opp_face(f)) {
          snprintf(why, whylen, "the mixed path needs neighbour face = opposite face");
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
      } else if (!same_geo(e[0], dcf) || !same_geo(e[1], inv_dcc) || !same_geo(e[2], area)) {
        snprintf(why, whylen, "the mixed path needs octree-regular geometry (cell %lld face %d)", (long long)c, f);
        return FVGPU_ERR_UNSUPPORTED;
      }
    }
    geom[size_t(c)] = code;
  }
  // bricks: same-level Morton blocks (candidates), kept when each of their
  // six sides is a domain boundary or another candidate block of the same
  // shape, whichever kernel evaluates that block (its cells only supply the
  // 2-deep halo).  8x8x4 bricks first; 4x4x4 bricks only on meshes where the
  // 8x8x4 ones cover under 5 % of the cells.  Where both exist, carving 4x4x4
  // blocks out of the general runs fragments them, and the general kernel's
  // cost per cell rises more than the bricks save (measured on the two-phase
  // bubble: 30 % fewer general cells, 4 % more general-kernel time).
  std::vector<char> is_block8(size_t(n), 0), is_brick8(size_t(n), 0), in_brick8(size_t(n), 0);
  std::vector<char> is_block4(size_t(n), 0), is_brick4(size_t(n), 0);
  // bricks for model 1, inviscid or viscous (both kernels read the cells'
  // gradients straight from the gradient pass); model 3 (paired state words,
  // float-float reconstruction of the partial densities) runs the general kernel
  if (!r.force_general && ph.model == 1) {
    find_blocks<Brick8>(m, is_block8);
    for (int64_t i = 0; i < n; ++i)
      if (is_block8[size_t(i)] && brick_sides_resolve<Brick8>(m, i, is_block8)) {
        is_brick8[size_t(i)] = 1;
        for (int t = 0; t < Brick8::N; ++t) in_brick8[size_t(i + t)] = 1;
      }
    int64_t covered8 = 0;
    for (int64_t i = 0; i < n; ++i) covered8 += in_brick8[size_t(i)];
    if (covered8 * 20 < n) {
      find_blocks<Brick4>(m, is_block4);
      for (int64_t i = 0; i < n; ++i)
        if (is_block4[size_t(i)] && !in_brick8[size_t(i)] && brick_sides_resolve<Brick4>(m, i, is_block4))
          is_brick4[size_t(i)] = 1;
    }
  }
  std::vector<BlockDesc> bricks, bricks4, general;
  auto brick_desc = [&](int64_t i, int count, auto side_of) {
    BlockDesc d;
    memset(&d, 0, sizeof d);
    d.start = int(i);
    d.count = count;
    d.level = m->level[i];
    for (int f = 0; f < 6; ++f) d.side[f] = side_of(f);
    return d;
  };
  for (int64_t i = 0; i < n;) {
    if (is_brick8[size_t(i)]) {
      bricks.push_back(brick_desc(i, Brick8::N, [&](int f) { return brick_side<Brick8>(m, i, f, is_block8); }));
      i += Brick8::N;
      continue;
    }
    if (is_brick4[size_t(i)]) {
      bricks4.push_back(brick_desc(i, Brick4::N, [&](int f) { return brick_side<Brick4>(m, i, f, is_block4); }));
      i += Brick4::N;
      continue;
    }
    BlockDesc d;
    memset(&d, 0, sizeof d);
    d.start = int(i);
    int cnt = 0;
    while (i < n && cnt < kBlock && !is_brick8[size_t(i)] && !is_brick4[size_t(i)]) {
      ++i;
      ++cnt;
    }
    d.count = cnt;
    general.push_back(d);
  }
  std::vector<BlockDesc> all(bricks);
  all.insert(all.end(), bricks4.begin(), bricks4.end());
  all.insert(all.end(), general.begin(), general.end());
  const int64_t nv = ph.model == 3 ? kNv<3> : kNv<1>;  // FP32 state words per cell
  r.geo_host.assign(reinterpret_cast<const unsigned char *>(&gt), reinterpret_cast<const unsigned char *>(&gt) + sizeof gt);
  cudaError_t e;
  if ((e = alloc_slot(r, kBufGeom, sizeof(int32_t) * n)) != cudaSuccess ||
      (e = cudaMemcpy(r.buf[kBufGeom], geom.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = alloc_slot(r, kBufTables, sizeof(GeoTables))) != cudaSuccess ||
      (e = cudaMemcpy(r.buf[kBufTables], &gt, sizeof gt, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = alloc_slot(r, kBufBlocks, sizeof(BlockDesc) * (all.size() + 1))) != cudaSuccess ||
      (e = cudaMemcpy(r.buf[kBufBlocks], all.data(), sizeof(BlockDesc) * all.size(), cudaMemcpyHostToDevice)) !=
          cudaSuccess ||
      (e = alloc_slot(r, kBufD1, sizeof(float) * kNeqMax * n)) != cudaSuccess ||
      (e = alloc_slot(r, kBufD2, sizeof(float) * kNeqMax * n)) != cudaSuccess ||
      (e = alloc_slot(r, kBufAlt, sizeof(double) * kNeqMax * n)) != cudaSuccess ||
      (e = alloc_slot(r, kBufSNf, sizeof(float) * nv * n)) != cudaSuccess ||
      (e = alloc_slot(r, kBufSNfAlt, sizeof(float) * nv * n)) != cudaSuccess ||
      (e = alloc_slot(r, kBufX1, sizeof(float) * nv * n)) != cudaSuccess ||
      (e = alloc_slot(r, kBufX2, sizeof(float) * nv * n)) != cudaSuccess ||
      (e = alloc_slot(r, kBufSG, ph.ns == 1 ? sizeof(float) * 9 * n : 16)) != cudaSuccess) {
    snprintf(why, whylen, "mixed-path allocation: %s", cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? FVGPU_ERR_NOMEM : FVGPU_ERR_CUDA;
  }
  r.n = n;
  r.model = ph.model;
  r.nbricks = int64_t(bricks.size());
  r.nbricks4 = int64_t(bricks4.size());
  r.ngeneral = int64_t(general.size());
  const int kinds = (r.nbricks > 0) + (r.nbricks4 > 0) + (r.ngeneral > 0);
  if (kinds > 1 && !r.side[0]) {
    for (int k = 0; k < 2; ++k)
      if (cudaStreamCreateWithFlags(&r.side[k], cudaStreamNonBlocking) != cudaSuccess ||
          cudaEventCreateWithFlags(&r.join_ev[k], cudaEventDisableTiming) != cudaSuccess) {
        snprintf(why, whylen, "stream / event creation failed");
        return FVGPU_ERR_CUDA;
      }
    if (cudaEventCreateWithFlags(&r.fork_ev, cudaEventDisableTiming) != cudaSuccess) {
      snprintf(why, whylen, "stream / event creation failed");
      return FVGPU_ERR_CUDA;
    }
  }
  r.ready = true;
  return FVGPU_OK;
}

void release_mixed(MixedResources &r) {
  for (int i = 0; i < 11; ++i) {
    if (r.buf[i]) cudaFree(r.buf[i]);
    r.buf[i] = nullptr;
    r.bytes[i] = 0;
    r.cap[i] = 0;
  }
  for (int k = 0; k < 2; ++k) {
    if (r.side[k]) cudaStreamDestroy(r.side[k]);
    if (r.join_ev[k]) cudaEventDestroy(r.join_ev[k]);
    r.side[k] = nullptr;
    r.join_ev[k] = nullptr;
  }
  if (r.fork_ev) cudaEventDestroy(r.fork_ev);
  r.fork_ev = nullptr;
  r.ready = false;
  r.snf_valid = false;
  r.nbricks = r.nbricks4 = r.ngeneral = 0;
}

cudaError_t mixed_refresh_f32(MixedResources &r, const double *S, int neq, LaunchMarks &marks, cudaStream_t st) {
  marks.mark(FVGPU_KIND_MIXED_AUX);
  if (r.model == 3)
    k_state_to_f32_m3<<<1024, 256, 0, st>>>(S, static_cast<float *>(r.buf[kBufSNf]), r.n);
  else
    k_state_to_f32<<<1024, 256, 0, st>>>(S, static_cast<float *>(r.buf[kBufSNf]), int64_t(neq) * r.n);
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) r.snf_valid = true;
  return e;
}

cudaError_t mixed_refresh_f32_lambda(MixedResources &r, const Phys &ph, const double *S, double *lambda,
                                     LaunchMarks &marks, cudaStream_t st) {
  marks.mark(FVGPU_KIND_MIXED_AUX);
  const unsigned blocks = unsigned(std::min<int64_t>((r.n + kBlock - 1) / kBlock, 152 * 8));
  const MixedConst mc = make_const(ph);
  const int32_t *geom = static_cast<const int32_t *>(r.buf[kBufGeom]);
  const GeoTables *geo = static_cast<const GeoTables *>(r.buf[kBufTables]);
  float *Sf = static_cast<float *>(r.buf[kBufSNf]);
  if (ph.model == 1)
    k_state_to_f32_lambda<1><<<blocks, kBlock, 0, st>>>(mc, geom, geo, S, Sf, int(r.n), lambda);
  else
    k_state_to_f32_lambda<3><<<blocks, kBlock, 0, st>>>(mc, geom, geo, S, Sf, int(r.n), lambda);
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) r.snf_valid = true;
  return e;
}

// the kernel instance of the configuration (EOS model, reconstruction order)
template <int MODEL, bool MUSCL, class S>
void launch_brick(unsigned grid, const MixedConst &mc, const StageArgs &a, cudaStream_t st) {
  static_assert(MODEL == 1, "bricks serve model 1");
  if (mc.ns == 1)
    k_mixed_brick<MODEL, MUSCL, true, S><<<grid, S::N, 0, st>>>(mc, a);
  else
    k_mixed_brick<MODEL, MUSCL, false, S><<<grid, S::N, 0, st>>>(mc, a);
}

enum BlockKind { kKindGeneral = 0, kKindBrick8 = 1, kKindBrick4 = 2 };

template <int MODEL, bool MUSCL>
void launch_instance(int kind, unsigned grid, const MixedConst &mc, const StageArgs &a, const GeoTables &geo,
                     cudaStream_t st) {
  if constexpr (MODEL == 1) {
    if (kind == kKindBrick8) return launch_brick<MODEL, MUSCL, Brick8>(grid, mc, a, st);
    if (kind == kKindBrick4) return launch_brick<MODEL, MUSCL, Brick4>(grid, mc, a, st);
  }
  k_mixed_general<MODEL, MUSCL><<<grid, kBlock, 0, st>>>(mc, a, geo);
}

void launch_kernel(const Phys &ph, int kind, unsigned grid, const MixedConst &mc, const StageArgs &a,
                   const GeoTables &geo, cudaStream_t st) {
  const bool muscl = ph.ischeme == 2;
  if (ph.model == 1)
    muscl ? launch_instance<1, true>(kind, grid, mc, a, geo, st) : launch_instance<1, false>(kind, grid, mc, a, geo, st);
  else
    muscl ? launch_instance<3, true>(kind, grid, mc, a, geo, st) : launch_instance<3, false>(kind, grid, mc, a, geo, st);
}

// One RK step from FP64 state `in` (and its FP32 copy) to `out`.
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
  float *X[2] = {static_cast<float *>(r.buf[kBufX1]), static_cast<float *>(r.buf[kBufX2])};
  const MixedConst mc = make_const(ph);
  const BlockDesc *blocks = static_cast<const BlockDesc *>(r.buf[kBufBlocks]);
  for (int k = 0; k < nst; ++k) {
    StageArgs a = stage_args(r, m);
    a.SNf = static_cast<const float *>(r.buf[kBufSNf]);
    a.Sin = k == 0 ? a.SNf : X[(k - 1) & 1];
    a.Din = k == 0 ? nullptr : D[(k - 1) & 1];
    a.Dout = D[k & 1];
    a.Sout = X[k & 1];
    a.SG = static_cast<const float *>(r.buf[kBufSG]);
    a.SN = in;
    a.SNout = out;
    a.SNfout = static_cast<float *>(r.buf[kBufSNfAlt]);
    a.dt = dt;
    a.irk = kStages[scheme][k];
    a.last = k == nst - 1;
    a.lambda = (a.last && cfl_mode) ? lambda : nullptr;
    a.err = err;
    if (ph.ns == 1) {
      marks.mark(FVGPU_KIND_MIXED_AUX);
      const unsigned gg = unsigned((m.n + kBlock - 1) / kBlock);
      if (ph.model == 1)
        k_mixed_grad<1><<<gg, kBlock, 0, st>>>(mc, a, static_cast<float *>(r.buf[kBufSG]),
                                               *reinterpret_cast<const GeoTables *>(r.geo_host.data()));
      else
        k_mixed_grad<3><<<gg, kBlock, 0, st>>>(mc, a, static_cast<float *>(r.buf[kBufSG]),
                                               *reinterpret_cast<const GeoTables *>(r.geo_host.data()));
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
    // the three kinds of block write disjoint cells: with more than one
    // present, 4x4x4 bricks and general blocks run on the side streams,
    // concurrently with the 8x8x4 bricks on the caller's stream
    const int64_t count[3] = {r.nbricks, r.nbricks4, r.ngeneral};
    const int64_t offset[3] = {0, r.nbricks, r.nbricks + r.nbricks4};
    const int kind_of[3] = {kKindBrick8, kKindBrick4, kKindGeneral};
    const bool fork = ((count[0] > 0) + (count[1] > 0) + (count[2] > 0)) > 1 && r.side[0];
    marks.mark(FVGPU_KIND_MIXED_STAGE);
    if (fork) {
      // only side streams that get work join (a captured stream must rejoin)
      cudaError_t e = cudaEventRecord(r.fork_ev, st);
      for (int k = 1; k < 3 && e == cudaSuccess; ++k)
        if (count[k] > 0) e = cudaStreamWaitEvent(r.side[k - 1], r.fork_ev, 0);
      if (e != cudaSuccess) return e;
    }
    for (int k = 2; k >= 0; --k) {  // side streams first, the caller's stream last
      if (count[k] == 0) continue;
      cudaStream_t ks = (fork && k > 0) ? r.side[k - 1] : st;
      a.blocks = blocks + offset[k];
      launch_kernel(ph, kind_of[k], unsigned(count[k]), mc, a, *reinterpret_cast<const GeoTables *>(r.geo_host.data()),
                    ks);
      cudaError_t e = cudaGetLastError();
      if (e == cudaSuccess && ks != st) e = cudaEventRecord(r.join_ev[k - 1], ks);
      if (e != cudaSuccess) return e;
    }
    if (fork) {
      for (int k = 1; k < 3; ++k) {
        if (count[k] == 0) continue;
        const cudaError_t e = cudaStreamWaitEvent(st, r.join_ev[k - 1], 0);
        if (e != cudaSuccess) return e;
      }
    }
  }
  return cudaSuccess;
}

}  // namespace amr
}  // namespace fv
