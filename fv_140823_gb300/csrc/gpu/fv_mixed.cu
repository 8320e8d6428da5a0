// fvbuild: -fmad=false
//
// FP32-mixed path: fused kernels per RK stage.
//
// Arithmetic.  Reconstruction, equation of state and HLLC fluxes run in FP32
// (model 3, in fv_mixed_amr.cu, keeps its density words and the mixture EOS
// inversion in float-float).  The state is kept in FP64
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
// Reconstruction.  minmod-limited MUSCL on the conservative variables
// (reconctruct_V3.c:17-43).  Where both faces of a cell on an axis have a
// same-level neighbour, the limited slope is one number per cell, axis and
// variable, s = minmod(q+ - q, q - q-) (the median of the two differences and
// zero), and the two face values are q +- k s with k = dist_cf / dist_cc of
// the level: the reference's slopes toward the two faces differ only through
// its dead band |d| > 1e-10, which this path drops (it moves a face value by
// at most k 1e-10).  Every other axis (a 1:4 face, a coarser neighbour, a
// domain boundary) keeps the reference's per-face form with the dead band.
//
// Canonical face fluxes.  Every face flux is defined from the face's lower
// cell (the one whose +x/+y/+z face it is), with that face's frame.  Whoever
// evaluates a face gets the same bits (this translation unit is compiled
// without automatic multiply-add contraction, explicit fmaf only), so the
// scheme is conservative and deterministic however the work is split.  A
// cell's residual is summed axis by axis, x, y, z: R += A (F- - F+) where
// neither face of the axis is a 1:4 face (a uniform flow cancels exactly),
// R += (T- - T+) with T the area-weighted sum over the sub-faces otherwise.
//
// Face frames are those of the reference's hexahedral cells (checked at
// upload), compiled in as signed permutations: rotating the momentum into
// and out of a face frame is a choice of registers.
//
// The kernel, k_mixed_brick, serves model-1 meshes that are Morton-aligned
// 8x8x4 bricks of same-level cells throughout (uniform octrees: the 128^3
// periodic case, the Sod tube), one brick per 256-thread block: the brick
// and its 2-deep face halo are staged in shared memory through constant
// index tables; each cell forms its six face values once (one slope per
// axis) and the halo cells next to the brick the one face value the brick
// needs; each thread then evaluates its cell's +x, +y, +z faces and the
// first threads the faces on the brick's lower sides; no neighbour tables
// are read; viscous runs read the two cells' gradients of each face.  Its
// tile and face-value slots live in dynamic shared memory (opted in above
// the 48 KiB default).  Every other mesh (AMR, model 3, FVGPU_FLAG_NO_BRICKS)
// runs the table-driven family of fv_mixed_amr.cu; the family is chosen
// once per mesh, so a context's results do not depend on how its cells are
// split into blocks.
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

namespace {

constexpr int kBlock = 256;
constexpr int kMaxLevel = 18;
constexpr int kRelSame = 0, kRelFiner = 1, kRelCoarser = 2, kRelBoundary = 3;
constexpr int kGeoStride = 4;  // per (level, face, relation): dcf, 1/dcc, area, k = dcf/dcc
constexpr int kGeoEntries = (kMaxLevel + 1) * 6 * 4;

struct GeoTables {
  float face[kGeoEntries * kGeoStride];
  float axis_area[(kMaxLevel + 1) * 3];  // area of a single-neighbour face normal to the axis
  float sub_area[(kMaxLevel + 1) * 6];
  float vol[kMaxLevel + 1];
  float inv_vol[kMaxLevel + 1];
  float inv2vol[kMaxLevel + 1];  // 1 / (2 V): CFL radius
};

__host__ __device__ constexpr int geo_index(int level, int f, int rel) { return ((level * 6 + f) * 4 + rel); }
// faces of an axis: + faces +x (1), +y (2), +z (5); - faces -x (3), -y (0), -z (4)
__host__ __device__ constexpr int plus_face(int a) { return a == 0 ? 1 : (a == 1 ? 2 : 5); }
__host__ __device__ constexpr int minus_face(int a) { return a == 0 ? 3 : (a == 1 ? 0 : 4); }
__host__ __device__ constexpr int axis_of_face(int f) { return (f == 1 || f == 3) ? 0 : ((f == 0 || f == 2) ? 1 : 2); }

// FP32 words of the state vector: the five conservative variables of
// model 1 (this file serves model 1; model 3 runs in fv_mixed_amr.cu).
template <int MODEL>
constexpr int kNv = 5;
constexpr int kNvMax = 5;
static_assert(kNvMax == kNeqMax, "model 1 state words");

// FP32 constants, converted once on the host.
struct MixedConst {
  float fr[54];  // face frames n, t1, t2 per face index
  float gamma, pinf, gm1, gpinf;
  float ylo, yhi;  // mass-fraction clip (facercnstr.c:43-44)
  float visc;      // dynamic viscosity (flux_viscous.c, turb = 0)
  int ns, eos;     // viscous fluxes on; energy work term on
  float inflow[kNvMax];  // conservative inflow ghost in FP32 state form
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
  const float *SNf;         // [nv][n] FP32 copy of the step-start state
  const float *Sin;         // [nv][n] FP32 stage-input state SNf + Din (SNf at the first stage)
  const float *Din;         // [5][n] stage-input increment (null: zero)
  float *Dout;              // [5][n]
  float *Sout;              // [nv][n] non-last stages: the next stage's input SNf + Dout
  const float *SG;          // [9][n] viscous runs: momentum gradients of Sin (ux uy uz vx ... wz)
  const double *SN;         // [neq][n] step-start state (last stage)
  double *SNout;            // [neq][n] last stage: SN + D
  float *SNfout;            // [nv][n] last stage: FP32 copy of SNout
  const double *dt;
  double *lambda;           // last stage: CFL radius of the new state
  int irk;
  int last;
  int ahead;  // the brick this many blocks ahead (one wave of resident blocks) gets its stage input prefetched
  unsigned long long *err;
};

// FP32 state arrays of this family (SNf, stage inputs, stage increments) are
// brick-major and cell-major within a brick: the 8x8x4 brick of cells
// [256 b, 256 b + 256) keeps one 5 KiB run, words 0-3 of its cells as 256
// float4 (word 0 of cell c at f4idx(c)), then word 4 of its cells (at
// f1idx(c)).  A cell's five words move with one 16-byte and one 4-byte
// access; a brick's stage data is one contiguous run.  (The FP64 state stays
// [neq][n], the layout of the C ABI.)
constexpr int kBrickCells = 256;
__host__ __device__ __forceinline__ int f4idx(int c) { return 4 * c + (c & ~(kBrickCells - 1)); }
__host__ __device__ __forceinline__ int f1idx(int c) { return c + 4 * (c & ~(kBrickCells - 1)) + 4 * kBrickCells; }
// the first float of the run of the brick that starts at cell b
__host__ __device__ __forceinline__ int brick_run(int b) { return 5 * b; }
__device__ __forceinline__ void ld5g(const float *p, int c, float q[5]) {
  const float4 u = __ldg(reinterpret_cast<const float4 *>(p + f4idx(c)));
  q[0] = u.x;
  q[1] = u.y;
  q[2] = u.z;
  q[3] = u.w;
  q[4] = __ldg(p + f1idx(c));
}
__device__ __forceinline__ void st5g(float *p, int c, const float q[5]) {
  *reinterpret_cast<float4 *>(p + f4idx(c)) = make_float4(q[0], q[1], q[2], q[3]);
  p[f1idx(c)] = q[4];
}

__device__ __forceinline__ int level_of(int32_t g) { return g & 31; }
__device__ __forceinline__ int rel_of(int32_t g, int f) { return (g >> (5 + 2 * f)) & 3; }
__device__ __forceinline__ const float *geo_face(const GeoTables *G, int level, int f, int rel) {
  return G->face + geo_index(level, f, rel) * kGeoStride;
}

// Hardware approximations (one special-function instruction each): relative
// error ~2^-22, far below the FP32 rounding the rest of the flux carries.
__device__ __forceinline__ float fast_rcp(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float fast_sqrt(float x) {
  float y;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
template <int MODEL>
__device__ __forceinline__ float state_rho(const float *q) { return q[0]; }
__device__ __forceinline__ float state_rho_rt(int, float q0) { return q0; }
// FP32 state words of an FP64 state
template <int MODEL>
__device__ __forceinline__ void to_state_f32(const double x[kNeqMax], float q[kNvMax]) {
#pragma unroll
  for (int v = 0; v < kNeqMax; ++v) q[v] = __double2float_rn(x[v]);
}

// d = a - b on the state words
template <int MODEL>
__device__ __forceinline__ void state_diff(const float a[kNvMax], const float b[kNvMax], float d[kNeqMax]) {
#pragma unroll
  for (int v = 0; v < kNeqMax; ++v) d[v] = a[v] - b[v];
}
// out = q + c s per variable (one fused multiply-add)
template <int MODEL>
__device__ __forceinline__ void add_slope(const float q[kNvMax], float c, const float s[kNeqMax], float out[kNvMax]) {
#pragma unroll
  for (int v = 0; v < kNeqMax; ++v) out[v] = fmaf(c, s[v], q[v]);
}

// FP32 face state in the Cartesian frame (facevalues.c:113-142): the CFL
// radius.
struct FS {
  float r, u, v, w, p, c;
};
template <int MODEL>
__device__ __forceinline__ bool mixed_face_state(const MixedConst &mc, const float *q, FS &s) {
  s.r = q[0];
  const float rinv = fast_rcp(s.r);
  s.u = q[1] * rinv;
  s.v = q[2] * rinv;
  s.w = q[3] * rinv;
  const float msq = fmaf(q[3], q[3], fmaf(q[2], q[2], q[1] * q[1]));
  s.p = fmaf(mc.gm1, fmaf(-0.5f * msq, rinv, q[4]), -mc.gpinf);
  s.c = fast_sqrt(fmaf(mc.gamma, s.p, mc.gpinf) * rinv);
  return true;
}

// Value across a boundary face (deltavalues.c:9-14; bc.c:19-49): the own
// state (transmissive), the inflow state, or the own state with the momentum
// mirrored as such (slip wall: normal component; no-slip wall: all of it),
// which on the axis-aligned faces is exact, as in the FP64 path.
template <int MODEL>
__device__ __forceinline__ void boundary_value(const MixedConst &mc, int bc, int f, const float own[kNvMax],
                                               float nb[kNvMax]) {
#pragma unroll
  for (int v = 0; v < kNvMax; ++v) nb[v] = own[v];
  if (bc == 1) {
#pragma unroll
    for (int v = 0; v < kNvMax; ++v) nb[v] = mc.inflow[v];
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
// tangents t1, t2), the normal velocity, pressure and sound speed.  The mixed
// path requires orthonormal frames (checked at upload), so |m|^2 and the
// stress contraction n.(p I).n = p are frame invariant; tangential velocities
// are formed only for the upwind state the HLLC flux takes.
struct LS {
  float r, rinv, mn, mm, ml;  // density, its reciprocal, local momentum
  float un;                   // normal velocity
  float p, c, e, y;           // pressure, sound speed, energy, (unused) mass fraction
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
__device__ __forceinline__ float frame_in_row(const float *q) {
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
__device__ __forceinline__ void frame_in_f(const float *q, float &mn, float &mm, float &ml) {
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
__device__ __forceinline__ void frame_in(int f, const float *q, float &mn, float &mm, float &ml) {
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
__device__ __forceinline__ bool local_state(const MixedConst &mc, int f, const float *q, bool, LS &s) {
  static_assert(MODEL == 1, "model 1 face states");
  frame_in<F>(f, q, s.mn, s.mm, s.ml);
  s.r = q[0];
  s.rinv = fast_rcp(s.r);
  s.un = s.mn * s.rinv;
  s.e = q[4];
  s.y = 0.0f;
  // p = (gamma - 1) (E - |m|^2 / (2 rho)) - gamma pinf, c^2 = gamma (p + pinf) / rho
  const float msq = fmaf(s.ml, s.ml, fmaf(s.mm, s.mm, s.mn * s.mn));
  s.p = fmaf(mc.gm1, fmaf(-0.5f * msq, s.rinv, s.e), -mc.gpinf);
  s.c = fast_sqrt(fmaf(mc.gamma, s.p, mc.gpinf) * s.rinv);
  return true;
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
  float S_S = num * fast_rcp(den);
  const bool ok = !isnan(S_S);
  if (bc == 3) S_S = 0.0f;
  // region selection of hllc_euler.c:18-50 (0 <= SL: left; SL <= 0 <= S*:
  // left star; S* <= 0 <= SR: right star; SR <= 0: right), reduced to two
  // predicates; with S* not NaN (NaN wave speeds make S* NaN) exactly one
  // region holds
  const bool gl = 0.0f <= SL, gs = 0.0f <= S_S, gr = 0.0f <= SR;
  const bool left = gl || gs;
  const bool star = !gl && (gs || gr);
  const float Kr = left ? L.r : R.r, Kmn = left ? L.mn : R.mn, Kun = left ? L.un : R.un;
  const float Kp = left ? L.p : R.p, Ke = left ? L.e : R.e, Ky = left ? L.y : R.y;
  const float Krinv = left ? L.rinv : R.rinv, Kmm = left ? L.mm : R.mm, Kml = left ? L.ml : R.ml;
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
  const float Fb = m * (Kmm * Krinv);
  const float Fc = m * (Kml * Krinv);
  const float F4 = MODEL == 1 ? (ee + pp) * un : m * Ky;
  Fn[0] = F0;
  frame_out<F>(f, Fa, Fb, Fc, Fn);
  Fn[4] = F4;
  return ok;
}

// Canonical flux of a face from the lower / upper face values (bc > 0: a
// domain-boundary face, the upper side is the ghost of the lower one).
template <int MODEL, int F = -1>
__device__ __forceinline__ bool canonical_flux(const MixedConst &mc, int f, int bc, bool clip, const float *lo,
                                               const float *hi, float Fn[kNeqMax]) {
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

// ============================ reconstruction ================================

// minmod of a and b: the one of smaller magnitude when both have the same
// sign, else zero.  min.xorsign.abs gives min(|a|, |b|) with the sign bit
// set when the signs differ; clamped at zero and given a's sign, that is the
// median of a, b and 0 up to the sign of a zero result.
__device__ __forceinline__ float minmod(float a, float b) {
  float m;
  asm("min.xorsign.abs.f32 %0, %1, %2;" : "=f"(m) : "f"(a), "f"(b));
  return copysignf(fmaxf(m, 0.0f), a);
}

// Face values of a cell on an axis whose two neighbours have the cell's
// level: s = minmod(q+ - q, q - q-), face+ = q + k s, face- = q - k s.
// WHICH: 1 only face+, -1 only face-, 0 both.
template <int MODEL, int WHICH = 0>
__device__ __forceinline__ void axis_faces(const float q[kNvMax], const float nbp[kNvMax], const float nbm[kNvMax],
                                           float k, float fp[kNvMax], float fm[kNvMax]) {
  float dp[kNeqMax], dm[kNeqMax], s[kNeqMax];
  state_diff<MODEL>(nbp, q, dp);
  state_diff<MODEL>(q, nbm, dm);
#pragma unroll
  for (int v = 0; v < kNeqMax; ++v) s[v] = minmod(dp[v], dm[v]);
  if (WHICH >= 0) add_slope<MODEL>(q, k, s, fp);
  if (WHICH <= 0) add_slope<MODEL>(q, -k, s, fm);
}

// The reference's per-face limited slope (reconctruct_V3.c:17-43, slopes
// divided by dist_cc as multiplications) from the delta across the face (d0)
// and across the opposite face (d1): zero unless the face is active (not a
// domain boundary), |d0| > 1e-10 and sm * sp > 0; then the slope of smaller
// magnitude.  A NaN product (a domain boundary behind the cell has 1/dist_cc
// = inf and a zero delta) gives zero, as in the reference.
__device__ __forceinline__ float minmod_slope(bool active, float d0, float d1, float inv_p, float inv_m) {
  const float sp = d0 * inv_p, sm = -d1 * inv_m;
  const float m = fabsf(sm) > fabsf(sp) ? sp : sm;
  return (active && fabsf(d0) > 1e-10f && sm * sp > 0.0f) ? m : 0.0f;
}

// Face value of a face of a cell in the reference's per-face form: values
// across the face (nbf) and across the opposite face (nbo), the face's
// dist_cf and 1/dist_cc (inv_p) and the opposite face's 1/dist_cc (inv_m).
template <int MODEL>
__device__ __forceinline__ void face_general(const float q[kNvMax], const float nbf[kNvMax], const float nbo[kNvMax],
                                             bool active, float dcf, float inv_p, float inv_m, float out[kNvMax]) {
  float d0[kNeqMax], d1[kNeqMax], s[kNeqMax];
  state_diff<MODEL>(nbf, q, d0);
  state_diff<MODEL>(nbo, q, d1);
#pragma unroll
  for (int v = 0; v < kNeqMax; ++v) s[v] = minmod_slope(active, d0[v], d1[v], inv_p, inv_m);
  add_slope<MODEL>(q, dcf, s, out);
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
__device__ __forceinline__ float cell_lambda_with(const MixedConst &mc, const float q[kNvMax], AreaFn area,
                                                  float inv2vol) {
  FS s;
  mixed_face_state<MODEL>(mc, q, s);
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
                                               const float q[kNvMax]) {
  const int lev = level_of(g);
  return cell_lambda_with<MODEL>(
      mc, q,
      [geo, g, lev](int f) {
        const int rel = rel_of(g, f);
        return rel == kRelFiner ? 4.0f * geo->sub_area[lev * 6 + f] : geo_face(geo, lev, f, rel)[2];
      },
      geo->inv2vol[lev]);
}

// RK stage update of one cell in increment form; FP64 state, FP32 copy and
// CFL radius at the last stage (qn receives the new FP32 state words).
template <int MODEL, int HD = -1, int LS = -1>  // stage has an input increment / is the last (-1: run time)
__device__ __forceinline__ bool stage_update(const StageArgs &a, int c, float dtv, const float R[kNeqMax], bool ok,
                                             float qn[kNvMax]) {
  const bool has_din = HD < 0 ? a.Din != nullptr : HD == 1;
  const bool last = LS < 0 ? a.last != 0 : LS == 1;
  const int n = a.n;
  bool finite = true;
#pragma unroll
  for (int v = 0; v < kNeqMax; ++v)
    if (!isfinite(R[v])) finite = false;
  if (!(ok && finite)) raise_error(a.err, ok ? kErrNonFinite : kErrRegion, c);
  // the stage-input increment, read again here rather than kept in
  // registers through the flux phase
  float din[kNeqMax] = {0.f, 0.f, 0.f, 0.f, 0.f};
  if (has_din) ld5g(a.Din, c, din);
  // stage weight w: D_k = w (D_in + dt/V R), RK(1) D1 = dt/V R as such
  const float w = a.irk == 2 ? 0.25f : (a.irk == 3 ? (2.0f / 3.0f) : 0.5f);
  const bool first = HD == 0 ? true : (HD == 1 ? false : a.irk == 1);
  float dn[kNeqMax];
#pragma unroll
  for (int v = 0; v < kNeqMax; ++v) {
    const float incr = dtv * R[v];
    dn[v] = first ? incr : w * (din[v] + incr);
  }
  if (last) {
    double snew[kNeqMax];
#pragma unroll
    for (int v = 0; v < kNeqMax; ++v) {
      snew[v] = __ldg(a.SN + v * n + c) + double(dn[v]);
      a.SNout[v * n + c] = snew[v];
    }
    to_state_f32<MODEL>(snew, qn);
    st5g(a.SNfout, c, qn);
    return true;
  }
  {
    float sn[kNvMax], x[kNvMax];
    ld5g(a.SNf, c, sn);
#pragma unroll
    for (int v = 0; v < kNeqMax; ++v) x[v] = sn[v] + dn[v];  // the value the next stage would form
    st5g(a.Dout, c, dn);
    st5g(a.Sout, c, x);
  }
  return false;
}

// stage state of any cell from global memory (SNf + D, written by the
// previous stage)
template <int MODEL>
__device__ __forceinline__ void global_state(const StageArgs &a, int x, float q[kNvMax]) {
  ld5g(a.Sin, x, q);
}

// ============================ viscous terms =================================

// Cartesian velocity of the ghost across a boundary face f (bc.c:19-49) from
// the own face values q.
__device__ __forceinline__ void ghost_velocity(const MixedConst &mc, int bc, int f, const float *q, float u[3]) {
  if (bc == 1) {
    const float rinv = fast_rcp(state_rho_rt(mc.model, mc.inflow[0]));
    u[0] = mc.inflow[1] * rinv;
    u[1] = mc.inflow[2] * rinv;
    u[2] = mc.inflow[3] * rinv;
    return;
  }
  const float rinv = fast_rcp(state_rho_rt(mc.model, q[0]));
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
__device__ __forceinline__ void viscous_normal(const MixedConst &mc, int f, int bc, const float *lo,
                                               const float *hi, const float gl[9], const float gh[9],
                                               float FVn[kNeqMax]) {
  float ul[3], uh[3];
  {
    const float rinv = fast_rcp(state_rho_rt(mc.model, lo[0]));
    ul[0] = lo[1] * rinv;
    ul[1] = lo[2] * rinv;
    ul[2] = lo[3] * rinv;
  }
  if (bc > 0) {
    ghost_velocity(mc, bc, f, lo, uh);
  } else {
    const float rinv = fast_rcp(state_rho_rt(mc.model, hi[0]));
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

// (F - FV).n of a face: the canonical flux minus the viscous normal flux,
// with the gradients of the face's lower and upper cells clo / chi
template <int MODEL, int F = -1>
__device__ __forceinline__ bool face_flux(const MixedConst &mc, const StageArgs &a, int f, int bc, bool clip,
                                          const float *lo, const float *hi, int clo, int chi, float Fn[kNeqMax]) {
  const bool ok = canonical_flux<MODEL, F>(mc, f, bc, clip, lo, hi, Fn);
  if (mc.ns == 1) {
    float gl[9], gh[9], FVn[kNeqMax];
    load_grad9f(a.SG, a.n, clo, gl);
    load_grad9f(a.SG, a.n, chi, gh);
    viscous_normal(mc, f, bc, lo, hi, gl, gh, FVn);
#pragma unroll
    for (int v = 0; v < kNeqMax; ++v) Fn[v] -= FVn[v];
  }
  return ok;
}

// Green-Gauss momentum gradients of the stage-input state (gradcalc.c:9-47,
// rows of rho u, rho v, rho w), FP32, one cell per thread.
template <int MODEL>
__global__ void __launch_bounds__(kBlock) k_mixed_grad(MixedConst mc, StageArgs a, float *__restrict__ SGout) {
  const int c = blockIdx.x * kBlock + threadIdx.x;
  const int n = a.n;
  if (c >= n) return;
  float q[kNvMax];
  global_state<MODEL>(a, c, q);
  const int32_t g = __ldg(a.geom + c);
  const int lev = level_of(g);
  const float inv_vol = a.geo->inv_vol[lev];
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
        ghost_velocity(mc, bc, f, q, u);
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
      add(m, geo_face(a.geo, lev, f, kRelBoundary)[2]);
    } else if (is_hanging(code)) {
      const int32_t *k = a.hang_nbr + 4 * hang_index(code);
      const float A = a.geo->sub_area[lev * 6 + f];
      for (int s = 0; s < 4; ++s) {
        const int ks = __ldg(k + s);
        const float4 u = __ldg(reinterpret_cast<const float4 *>(a.Sin + f4idx(ks)));
        const float m[3] = {u.y, u.z, u.w};
        add(m, A);
      }
    } else {
      const float4 u = __ldg(reinterpret_cast<const float4 *>(a.Sin + f4idx(code)));
      const float m[3] = {u.y, u.z, u.w};
      add(m, geo_face(a.geo, lev, f, rel_of(g, f))[2]);
    }
  }
#pragma unroll
  for (int i = 0; i < 9; ++i) SGout[i * n + c] = gr[i];
}

// Slots of five FP32 words in shared memory: words 0-3 as one float4 and
// word 4 in a float array beside it, so that a slot moves with two
// shared-memory instructions.
struct Slots5 {
  float4 *p4;
  float *p1;
  __device__ __forceinline__ void ld(int i, float q[kNvMax]) const {
    const float4 u = p4[i];
    q[0] = u.x;
    q[1] = u.y;
    q[2] = u.z;
    q[3] = u.w;
    q[4] = p1[i];
  }
  __device__ __forceinline__ void st(int i, const float q[kNvMax]) const {
    p4[i] = make_float4(q[0], q[1], q[2], q[3]);
    p1[i] = q[4];
  }
};

// dynamic shared memory of the kernels (16-byte aligned)
extern __shared__ __align__(16) float g_mixed_smem[];

// 16-byte asynchronous global -> shared copy (cp.async.cg: L2 only)
__device__ __forceinline__ void cp_async16(float4 *dst, const float *src) {
  const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
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
// Face-value slots (the values a thread hands to another): the brick cells'
// -x, -y, -z face values (axis * N + t), then the halo cells next to the
// brick (layer 1), side by side in the order -x, +x, -y, +y, -z, +z.
template <int BX_, int BY_, int BZ_, int PAD_>
struct BrickShape {
  static constexpr int BX = BX_, BY = BY_, BZ = BZ_, N = BX_ * BY_ * BZ_;
  static constexpr int TX = BX + 4, TY = BY + 4, TZ = BZ + 4;
  static constexpr int P = TX * TY + PAD_;  // z-plane stride of the tile
  static constexpr int kTile = P * TZ;
  static constexpr int kFaces = (BX + 1) * BY * BZ + BX * (BY + 1) * BZ + BX * BY * (BZ + 1);
  static constexpr int kHalo = 2 * (2 * BY * BZ + 2 * BX * BZ + 2 * BX * BY);
  static constexpr int kHalo1 = 2 * (BY * BZ + BX * BZ + BX * BY);
  static constexpr int kSides = BY * BZ + BX * BZ + BX * BY;
  static constexpr int kFvSlots = 3 * N + kHalo1;
  // flux slots: the +x, +y, +z faces of the N cells (axis * N + t), then
  // the faces on the brick's -x, -y, -z sides
  static constexpr int kSlotSideX = 3 * N, kSlotSideY = kSlotSideX + BY * BZ, kSlotSideZ = kSlotSideY + BX * BZ;
  // blocks per SM the launch bounds ask for: inviscid 48 registers (five
  // 256-thread blocks), viscous 64 (four).  Neither spills.
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
  // layer-1 halo cell beyond brick side `side` at in-plane position (i, j):
  // (y, z) for the x sides, (x, z) for the y sides, (x, y) for the z sides
  __host__ __device__ static constexpr int halo1_index(int side, int i, int j) {
    return side == 3   ? i + BY * j
           : side == 1 ? BY * BZ + i + BY * j
           : side == 0 ? 2 * BY * BZ + i + BX * j
           : side == 2 ? 2 * BY * BZ + BX * BZ + i + BX * j
           : side == 4 ? 2 * BY * BZ + 2 * BX * BZ + i + BX * j
                       : 2 * BY * BZ + 2 * BX * BZ + BX * BY + i + BX * j;
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
  // dynamic shared memory: the tile (stage states, later the face fluxes)
  // and the face-value slots
  template <int NV>
  static constexpr size_t smem_bytes() { return sizeof(float) * NV * (kTile + kFvSlots); }
  static_assert(kTile <= 2048 && kFvSlots <= 1024 && kFaces <= 1024 && kSlotSideZ + BX * BY == kFaces &&
                    N <= 256 && BY % 2 == 0 && kNeqMax * kFaces <= 5 * kTile,
                "brick table fields");
};
using Brick8 = BrickShape<8, 8, 4, 2>;

// lower cell (brick coordinates) and axis of flux slot `slot`
template <class S>
__host__ __device__ constexpr void slot_lower_cell(int slot, int &axis, int &lx, int &ly, int &lz) {
  axis = 0;
  if (slot < S::kSlotSideX) {
    axis = slot / S::N;
    const int t = slot % S::N;
    lx = morton_x(t);
    ly = morton_y(t);
    lz = morton_z(t);
  } else if (slot < S::kSlotSideY) {
    const int r = slot - S::kSlotSideX;
    lx = -1;
    ly = r % S::BY;
    lz = r / S::BY;
  } else if (slot < S::kSlotSideZ) {
    const int r = slot - S::kSlotSideY;
    axis = 1;
    lx = r % S::BX;
    ly = -1;
    lz = r / S::BX;
  } else {
    const int r = slot - S::kSlotSideZ;
    axis = 2;
    lx = r % S::BX;
    ly = S::zslot_y(r);
    lz = -1;
  }
}

// The two cells of each flux slot (S::cell_ref), 12 bits each, lower first
// (viscous runs).
template <class S>
struct BrickTaskCells {
  uint32_t c[S::kFaces];
};
template <class S>
constexpr BrickTaskCells<S> make_brick_task_cells() {
  BrickTaskCells<S> C{};
  for (int slot = 0; slot < S::kFaces; ++slot) {
    int axis = 0, lx = 0, ly = 0, lz = 0;
    slot_lower_cell<S>(slot, axis, lx, ly, lz);
    C.c[slot] = S::cell_ref(lx, ly, lz) | (S::cell_ref(lx + (axis == 0), ly + (axis == 1), lz + (axis == 2)) << 12);
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
          bank_of[k] = ti % 8;  // 16-byte slots: eight per 128-byte wavefront
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

// Brick cells in Morton order, three words each.  Word 0: tile index (11
// bits), edge mask (6); word 1: flux slots of the cell's -x, -y, -z faces (10
// bits each; the +x, +y, +z faces are slots t, N + t, 2N + t); word 2:
// face-value slots of the upper cells across the +x, +y, +z faces (their
// - face values).
template <class S>
struct BrickCells {
  uint32_t w[3 * S::N];
};
template <class S>
constexpr BrickCells<S> make_brick_cells() {
  BrickCells<S> C{};
  constexpr int N = S::N;
  for (int t = 0; t < N; ++t) {
    const int x = morton_x(t), y = morton_y(t), z = morton_z(t);
    const int mx = x > 0 ? morton_local(x - 1, y, z) : S::kSlotSideX + y + S::BY * z;
    const int my = y > 0 ? N + morton_local(x, y - 1, z) : S::kSlotSideY + x + S::BX * z;
    const int mz = z > 0 ? 2 * N + morton_local(x, y, z - 1) : S::kSlotSideZ + S::zslot(x, y);
    const int px = x < S::BX - 1 ? morton_local(x + 1, y, z) : 3 * N + S::halo1_index(1, y, z);
    const int py = y < S::BY - 1 ? N + morton_local(x, y + 1, z) : 3 * N + S::halo1_index(2, x, z);
    const int pz = z < S::BZ - 1 ? 2 * N + morton_local(x, y, z + 1) : 3 * N + S::halo1_index(5, x, y);
    C.w[3 * t] = uint32_t(S::tile_index(x, y, z)) | (S::edge_mask(x, y, z) << 11);
    C.w[3 * t + 1] = uint32_t(mx) | (uint32_t(my) << 10) | (uint32_t(mz) << 20);
    C.w[3 * t + 2] = uint32_t(px) | (uint32_t(py) << 10) | (uint32_t(pz) << 20);
  }
  return C;
}
template <class S>
__device__ const BrickCells<S> g_brick_cells = make_brick_cells<S>();

// Layer-1 halo cells in face-value slot order.  Packed: tile index (11
// bits), axis (2), upper side (1: the cell's - face value is needed, else
// its + face value), brick side (3).
template <class S>
struct BrickHalo1 {
  uint32_t h[S::kHalo1];
};
template <class S>
constexpr BrickHalo1<S> make_brick_halo1() {
  BrickHalo1<S> H{};
  const int sides[6] = {3, 1, 0, 2, 4, 5};
  for (int k = 0; k < 6; ++k) {
    const int side = sides[k];
    const int axis = (side == 1 || side == 3) ? 0 : ((side == 0 || side == 2) ? 1 : 2);
    const bool upper = side == 1 || side == 2 || side == 5;
    const int ni = axis == 0 ? S::BY : S::BX, nj = axis == 2 ? S::BY : S::BZ;
    const int o = upper ? (axis == 0 ? S::BX : (axis == 1 ? S::BY : S::BZ)) : -1;
    for (int j = 0; j < nj; ++j)
      for (int i = 0; i < ni; ++i) {
        const int x = axis == 0 ? o : i, y = axis == 0 ? i : (axis == 1 ? o : j), z = axis == 2 ? o : j;
        H.h[S::halo1_index(side, i, j)] = uint32_t(S::tile_index(x, y, z)) | (uint32_t(axis) << 11) |
                                          (uint32_t(upper) << 13) | (uint32_t(side) << 14);
      }
  }
  return H;
}
template <class S>
__device__ const BrickHalo1<S> g_brick_halo1 = make_brick_halo1<S>();

// Faces on the brick's lower sides, in flux-slot order (slot 3N + j).
// Packed: face-value slot of the lower (halo) cell's + face value (10 bits),
// of the upper (brick) cell's - face value (10), axis (2).
template <class S>
struct BrickSides {
  uint32_t s[S::kSides];
};
template <class S>
constexpr BrickSides<S> make_brick_sides() {
  BrickSides<S> T{};
  constexpr int N = S::N;
  for (int j = 0; j < S::kSides; ++j) {
    int axis = 0, lx = 0, ly = 0, lz = 0;
    slot_lower_cell<S>(3 * N + j, axis, lx, ly, lz);
    int lo = 0, hi = 0;
    if (axis == 0) {
      lo = 3 * N + S::halo1_index(3, ly, lz);
      hi = morton_local(0, ly, lz);
    } else if (axis == 1) {
      lo = 3 * N + S::halo1_index(0, lx, lz);
      hi = N + morton_local(lx, 0, lz);
    } else {
      lo = 3 * N + S::halo1_index(4, lx, ly);
      hi = 2 * N + morton_local(lx, ly, 0);
    }
    T.s[j] = uint32_t(lo) | (uint32_t(hi) << 10) | (uint32_t(axis) << 20);
  }
  return T;
}
template <class S>
__device__ const BrickSides<S> g_brick_sides = make_brick_sides<S>();

// CFL radius of a brick cell: the frames are axis-aligned (checked at
// upload), so |u.n| on face f is the magnitude of one velocity component --
// the same value cell_lambda_with forms from the frame, without it.
template <int MODEL>
__device__ __forceinline__ float brick_lambda(const MixedConst &mc, const float q[kNvMax], uint32_t be,
                                              const float (*geo)[2][4], float inv2vol) {
  FS s;
  mixed_face_state<MODEL>(mc, q, s);
  const float au = fabsf(s.u), av = fabsf(s.v), aw = fabsf(s.w);
  float acc = 0.0f;
#pragma unroll
  for (int f = 0; f < 6; ++f) {
    const float un = (f == 1 || f == 3) ? au : ((f == 0 || f == 2) ? av : aw);
    acc = fmaf(geo[f][(be >> f) & 1u][2], un + s.c, acc);
  }
  return acc * inv2vol;
}

// One instance per stage kind: HD = 1 when the stage has an input increment
// (every stage but the first), LS = 1 for the last stage of the step (FP64
// update, FP32 copy, CFL radius); the kind's branches are resolved at
// compile time.
template <int MODEL, bool MUSCL, bool NS, class S, int HD, int LS>
__global__ void __launch_bounds__(S::N, NS ? S::kMinBlocksNS : S::kMinBlocks)
    k_mixed_brick(MixedConst mc, StageArgs a) {
  constexpr bool kHasDin = HD == 1, kLast = LS == 1;
  constexpr int NV = kNv<MODEL>;
  constexpr int TX = S::TX, NB = S::N;
  constexpr int kTile = S::kTile, kFaces = S::kFaces, kHalo = S::kHalo, kHalo1 = S::kHalo1;
  constexpr int kSides = S::kSides, kFvSlots = S::kFvSlots;
  // the tile holds the stage state of the brick and its halo until every
  // face value is formed, then the face fluxes (five-word slots)
  static_assert(kTile % 4 == 0, "float4 tile");
  const Slots5 tile{reinterpret_cast<float4 *>(g_mixed_smem), g_mixed_smem + 4 * kTile};
  static_assert(NV == 5 && (NV * kTile) % 4 == 0, "five-word slots, 16-byte aligned");
  const Slots5 fvb{reinterpret_cast<float4 *>(g_mixed_smem + NV * kTile),
                   g_mixed_smem + NV * kTile + 4 * kFvSlots};  // face values handed on
  const Slots5 flux{reinterpret_cast<float4 *>(g_mixed_smem), g_mixed_smem + 4 * kFaces};
  __shared__ float s_geo[6][2][4];  // per face index, relation same / boundary: dcf, 1/dcc, area, k
  __shared__ float s_area[3];       // face area per axis
  __shared__ float s_dtv, s_inv2vol;  // dt / V and 1 / (2 V) of the brick's level
  __shared__ int s_side[6];  // brick sides (indexed at run time: kept out of local memory)
  const BlockDesc *bdp = a.blocks + blockIdx.x;
  const int t = threadIdx.x;
  const int n = a.n;
  const int start = __ldg(&bdp->start), level = __ldg(&bdp->level);
  const int c = start + t;
  // lane f < 6 of every warp holds brick side f (the halo loop reads it by
  // shuffle); the sides on the domain boundary as a bit mask
  const int lane_side = __ldg(&bdp->side[(t & 31) < 6 ? (t & 31) : 0]);
  const uint32_t bmask = __ballot_sync(0xffffffffu, (t & 31) < 6 && lane_side < 0);
  if (t < 6) s_side[t] = lane_side;
  if (t < 12) {
    const int f = t >> 1, r = t & 1;
    const float *gf = geo_face(a.geo, level, f, r ? kRelBoundary : kRelSame);
#pragma unroll
    for (int k = 0; k < 4; ++k) s_geo[f][r][k] = gf[k];
  }
  if (t >= 12 && t < 15) s_area[t - 12] = a.geo->axis_area[level * 3 + (t - 12)];
  if (t == 0) {
    s_dtv = __double2float_rn(*a.dt) * a.geo->inv_vol[level];
    s_inv2vol = a.geo->inv2vol[level];
  }

  // the arrays the update reads at the end, on their way to L2 (128-byte
  // lines: NB / 16 per FP64 variable, NB / 32 per FP32 one)
  constexpr int kL64 = NB / 16, kL32 = NB / 32;
  if (kLast && t < kNeqMax * kL64) {  // the FP64 step-start state
    const int v = t / kL64, l = t % kL64;
    asm volatile("prefetch.global.L2 [%0];" ::"l"(a.SN + int64_t(v) * n + start + 16 * l));
  }
  if (kHasDin && t >= kNeqMax * kL64 && t < kNeqMax * (kL64 + kL32)) {  // the stage-input increment
    const int r = t - kNeqMax * kL64, v = r / kL32, l = r % kL32;
    asm volatile("prefetch.global.L2 [%0];" ::"l"(a.Din + brick_run(start) + kBrickCells * v + 32 * l));
  }
  if (kHasDin && !kLast && t >= kNeqMax * (kL64 + kL32) && t < kNeqMax * (kL64 + 2 * kL32)) {  // FP32 SN
    const int r = t - kNeqMax * (kL64 + kL32), v = r / kL32, l = r % kL32;
    asm volatile("prefetch.global.L2 [%0];" ::"l"(a.SNf + brick_run(start) + kBrickCells * v + 32 * l));
  }
  static_assert(kNeqMax * (kL64 + 2 * kL32) <= NB, "prefetch lanes");
  // the stage input of the brick one wave of resident blocks ahead, on its
  // way to L2 by the time that block starts
  if (a.ahead > 0 && int(blockIdx.x) + a.ahead < int(gridDim.x) && t >= NB - NV * kL32) {
    const int r = t - (NB - NV * kL32), v = r / kL32, l = r % kL32;
    const int next = __ldg(&a.blocks[blockIdx.x + a.ahead].start);
    asm volatile("prefetch.global.L2 [%0];" ::"l"(a.Sin + brick_run(next) + kBrickCells * v + 32 * l));
  }
  static_assert(NV * kL32 + kNeqMax * (kL64 + 2 * kL32) <= NB, "prefetch lanes do not overlap");
  // 1: the brick's cells and the halo from the six neighbour bricks, copied
  // global -> shared asynchronously (cp.async, no register round trip)
  const uint32_t cw0 = __ldg(&g_brick_cells<S>.w[3 * t]);
  const int ti = int(cw0 & 2047u);
  cp_async16(tile.p4 + ti, a.Sin + f4idx(c));
  cp_async4(tile.p1 + ti, a.Sin + f1idx(c));
#pragma unroll
  for (int h = t; h < kHalo; h += NB) {
    const uint32_t e = __ldg(&g_brick_halo<S>.h[h]);
    static_assert(kHalo % NB == 0, "every lane takes part in the side shuffle");
    static_assert(S::N == kBrickCells, "brick-major FP32 arrays hold 256-cell bricks");
    const int base = __shfl_sync(0xffffffffu, lane_side, int((e >> 11) & 7u));
    if (base >= 0) {
      const int hti = int(e & 2047u), x = base + int(e >> 14);
      cp_async16(tile.p4 + hti, a.Sin + f4idx(x));
      cp_async4(tile.p1 + hti, a.Sin + f1idx(x));
    }
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
  __syncthreads();
  // ghost values beyond domain-boundary sides (deltavalues.c:9-14): the
  // ghost of the brick cell next to it, in both halo layers
  if (bmask) {
#pragma unroll 1
    for (int h = t; h < kHalo1; h += NB) {
      const uint32_t e = __ldg(&g_brick_halo1<S>.h[h]);
      const int side = int((e >> 14) & 7u);
      if (!((bmask >> side) & 1u)) continue;
      const int ax = int((e >> 11) & 3u);
      const int st = ax == 0 ? 1 : (ax == 1 ? TX : S::P);
      const int sg = ((e >> 13) & 1u) ? st : -st;  // outward step
      const int h1 = int(e & 2047u), own_ti = h1 - sg;
      float own[kNvMax], gv[kNvMax];
      tile.ld(own_ti, own);
      boundary_value<MODEL>(mc, -1 - s_side[side], side, own, gv);
      tile.st(h1, gv);
      tile.st(h1 + sg, gv);
    }
    __syncthreads();  // bmask is uniform across the block
  }

  const uint32_t cw2 = __ldg(&g_brick_cells<S>.w[3 * t + 2]);
  auto cell_of = [&](uint32_t r) -> int {
    return (r & 2048u) ? s_side[(r >> 8) & 7u] + int(r & 255u) : start + int(r & 255u);
  };
  bool ok = true;
  const uint32_t be = (cw0 >> 11) & 63u & bmask;
  // 2-3 for a brick off the domain boundary (EDGE false) or on it
  auto body = [&](auto edge) {
    constexpr bool EDGE = decltype(edge)::value;
    // 2: face values.  Own cell: all six (one slope per axis); the + face
    // values stay in registers, the - face values go to the slots.
    float q[kNvMax];
    tile.ld(ti, q);
    float fpv[3][kNvMax];
    auto own_axis = [&](auto axc) {
      constexpr int AX = decltype(axc)::value;
      constexpr int FP = plus_face(AX), FM = minus_face(AX);
      constexpr int ST = AX == 0 ? 1 : (AX == 1 ? TX : S::P);
      float nbp[kNvMax], nbm[kNvMax], fm[kNvMax];
      tile.ld(ti + ST, nbp);
      tile.ld(ti - ST, nbm);
      if (!MUSCL) {
#pragma unroll
        for (int v = 0; v < kNvMax; ++v) fpv[AX][v] = fm[v] = q[v];
      } else if (EDGE && (be & ((1u << FP) | (1u << FM)))) {
        const int rp = (be >> FP) & 1u, rm = (be >> FM) & 1u;
        face_general<MODEL>(q, nbp, nbm, !rp, s_geo[FP][rp][0], s_geo[FP][rp][1], s_geo[FM][rm][1], fpv[AX]);
        face_general<MODEL>(q, nbm, nbp, !rm, s_geo[FM][rm][0], s_geo[FM][rm][1], s_geo[FP][rp][1], fm);
      } else {
        axis_faces<MODEL>(q, nbp, nbm, s_geo[FP][0][3], fpv[AX], fm);
      }
      fvb.st(AX * NB + t, fm);
    };
    own_axis(std::integral_constant<int, 0>{});
    own_axis(std::integral_constant<int, 1>{});
    own_axis(std::integral_constant<int, 2>{});
    // layer-1 halo cells: the one face value the brick needs
#pragma unroll
    for (int h = t; h < kHalo1; h += NB) {
      const uint32_t e = __ldg(&g_brick_halo1<S>.h[h]);
      if (!EDGE || !((bmask >> ((e >> 14) & 7u)) & 1u)) {
        const int hti = int(e & 2047u), ax = int((e >> 11) & 3u);
        const bool upper = (e >> 13) & 1u;
        const int st = ax == 0 ? 1 : (ax == 1 ? TX : S::P);
        float qh[kNvMax], nbp[kNvMax], nbm[kNvMax], out[kNvMax];
        tile.ld(hti, qh);
        tile.ld(hti + st, nbp);
        tile.ld(hti - st, nbm);
        if (!MUSCL) {
#pragma unroll
          for (int v = 0; v < kNvMax; ++v) out[v] = qh[v];
        } else {
          const float k = s_geo[plus_face(ax)][0][3];
          if (upper)
            axis_faces<MODEL, -1>(qh, nbp, nbm, k, out, out);
          else
            axis_faces<MODEL, 1>(qh, nbp, nbm, k, out, out);
        }
        fvb.st(3 * NB + h, out);
      }
    }
    __syncthreads();  // the tile is read for the last time above; it now takes the fluxes

    // 3: fluxes of the own + faces and of the faces on the brick's lower sides
    auto own_flux = [&](auto axc) {
      constexpr int AX = decltype(axc)::value;
      constexpr int FP = plus_face(AX);
      float Fn[kNeqMax];
      const int slot = AX * NB + t;
      if (EDGE && ((be >> FP) & 1u)) {  // the cell's own domain-boundary face (residual_faces_AMR.c:196-209)
        ok &= face_flux<MODEL, FP>(mc, a, FP, -1 - s_side[FP], MUSCL, fpv[AX], fpv[AX], c, c, Fn);
      } else {
        float hi[kNvMax];
        const int hs = int((cw2 >> (10 * AX)) & 1023u);
        fvb.ld(hs, hi);
        int clo = c, chi = c;
        if (NS) {
          const uint32_t cr = __ldg(&g_brick_task_cells<S>.c[slot]);
          clo = cell_of(cr & 4095u);
          chi = cell_of(cr >> 12);
        }
        ok &= face_flux<MODEL, FP>(mc, a, FP, 0, MUSCL, fpv[AX], hi, clo, chi, Fn);
      }
      flux.st(slot, Fn);
    };
    own_flux(std::integral_constant<int, 0>{});
    own_flux(std::integral_constant<int, 1>{});
    own_flux(std::integral_constant<int, 2>{});
#pragma unroll 1
    for (int j = t; j < kSides; j += NB) {
      const uint32_t e = __ldg(&g_brick_sides<S>.s[j]);
      const int ax = int((e >> 20) & 3u);
      const int fm = minus_face(ax);
      float Fn[kNeqMax], lo[kNvMax], hi[kNvMax];
      const int los = int(e & 1023u), his = int((e >> 10) & 1023u);
      fvb.ld(his, hi);
      if (EDGE && ((bmask >> fm) & 1u)) {
        // the brick cell's own domain-boundary face, own frame, stored as the
        // + face flux of the lower cell that is not there
        const int cown = start + his % NB;
        ok &= face_flux<MODEL>(mc, a, fm, -1 - s_side[fm], MUSCL, hi, hi, cown, cown, Fn);
#pragma unroll
        for (int v = 0; v < kNeqMax; ++v) Fn[v] = -Fn[v];
      } else {
        fvb.ld(los, lo);
        int clo = c, chi = c;
        if (NS) {
          const uint32_t cr = __ldg(&g_brick_task_cells<S>.c[3 * NB + j]);
          clo = cell_of(cr & 4095u);
          chi = cell_of(cr >> 12);
        }
        if (ax == 0)
          ok &= face_flux<MODEL, 1>(mc, a, 1, 0, MUSCL, lo, hi, clo, chi, Fn);
        else if (ax == 1)
          ok &= face_flux<MODEL, 2>(mc, a, 2, 0, MUSCL, lo, hi, clo, chi, Fn);
        else
          ok &= face_flux<MODEL, 5>(mc, a, 5, 0, MUSCL, lo, hi, clo, chi, Fn);
      }
      flux.st(3 * NB + j, Fn);
    }
  };
  if (bmask)
    body(std::true_type{});
  else
    body(std::false_type{});
  __syncthreads();

  // 4: residual axis by axis, x, y, z: R += A (F- - F+), then the RK stage update
  const uint32_t cw1 = __ldg(&g_brick_cells<S>.w[3 * t + 1]);
  float R[kNeqMax] = {0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) {
    const int sm = int((cw1 >> (10 * ax)) & 1023u), sp = ax * NB + t;
    const float A = s_area[ax];
    float fm[kNvMax], fp[kNvMax];
    flux.ld(sm, fm);
    flux.ld(sp, fp);
#pragma unroll
    for (int v = 0; v < kNeqMax; ++v) R[v] = fmaf(A, fm[v] - fp[v], R[v]);
  }
  float qn[kNvMax], lam = 0.0f;
  if (stage_update<MODEL, HD, LS>(a, c, s_dtv, R, ok, qn) && a.lambda)
    lam = brick_lambda<MODEL>(mc, qn, be, s_geo, s_inv2vol);
  if (kLast && a.lambda) block_max_lambda_f<NB>(lam, a.lambda);
}

// FP32 state words of an FP64 state (after an upload or an FP64-path
// step), one cell per thread.
template <int MODEL>
__global__ void k_state_to_f32(const double *__restrict__ S, float *__restrict__ Sf, int64_t n, int neq) {
  for (int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; c < n; c += int64_t(gridDim.x) * blockDim.x) {
    double x[kNeqMax];
#pragma unroll
    for (int v = 0; v < kNeqMax; ++v) x[v] = v < neq ? S[v * n + c] : 0.0;
    float q[kNvMax];
    to_state_f32<MODEL>(x, q);
    st5g(Sf, int(c), q);
  }
}

// The same with the CFL spectral radius of the copied state (the mixed
// path's first CFL time step after an upload).
template <int MODEL>
__global__ void __launch_bounds__(kBlock) k_state_to_f32_lambda(MixedConst mc, const int32_t *__restrict__ geom,
                                                                const GeoTables *geo, const double *__restrict__ S,
                                                                float *__restrict__ Sf, int n, double *lambda) {
  float lam = 0.0f;
  for (int c = blockIdx.x * kBlock + threadIdx.x; c < n; c += gridDim.x * kBlock) {
    double x[kNeqMax];
#pragma unroll
    for (int v = 0; v < kNeqMax; ++v) x[v] = v < mc.neq ? S[int64_t(v) * n + c] : 0.0;
    float q[kNvMax];
    to_state_f32<MODEL>(x, q);
    st5g(Sf, c, q);
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
  for (int v = 0; v < kNeqMax; ++v) mc.inflow[v] = float(ph.inflow[v]);
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

// every cell of a model-1 mesh lies in an 8x8x4 brick whose six sides are
// bricks or domain boundaries
bool all_cells_in_bricks(const fvgpu_mesh_soa *m, std::vector<char> &is_block8) {
  const int64_t n = m->ncells;
  if (n % Brick8::N != 0) return false;
  find_blocks<Brick8>(m, is_block8);
  for (int64_t i = 0; i < n; i += Brick8::N)
    if (!is_block8[size_t(i)] || !brick_sides_resolve<Brick8>(m, i, is_block8)) return false;
  return true;
}

}  // namespace

bool mixed_supported(const Phys &ph, char *why, size_t whylen) {
  if (ph.model != 1 && ph.model != 3) {
    snprintf(why, whylen, "the mixed path implements models 1 and 3");
    return false;
  }
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

// The kernel family of a mesh: the brick kernel of this file for model 1 in
// 8x8x4 bricks throughout, the table-driven family (fv_mixed_amr.cu)
// otherwise.
cudaError_t allow_smem_brick(bool muscl, bool ns);  // with the launches below

// resident brick blocks across the GPU (the prefetch distance of the stage input)
int brick_wave(bool muscl, bool ns);

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
  std::vector<char> is_block8(size_t(m->ncells), 0);
  if (ph.model != 1 || r.force_general || !all_cells_in_bricks(m, is_block8)) {
    r.family = 1;
    return amr::mixed_prepare_host(r, ph, m, why, whylen);
  }
  if (m->ncells > (int64_t(INT_MAX) - kBrickCells) / 5) {
    snprintf(why, whylen, "the mixed path indexes its FP32 arrays with 32-bit integers: at most %lld cells",
             (long long)((int64_t(INT_MAX) - kBrickCells) / 5));
    return FVGPU_ERR_UNSUPPORTED;
  }
  r.family = 0;
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
  std::vector<char> seen_axis((kMaxLevel + 1) * 3, 0);
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
      // the slope factor dist_cf / dist_cc of a face between two same-level cells
      const float kf = rel == kRelSame ? float(m->dcf[i] / m->dcc[i]) : 0.0f;
      const int gi = geo_index(lev, f, rel);
      float *e = gt.face + gi * kGeoStride;
      if (!seen[gi]) {
        seen[gi] = 1;
        e[0] = dcf;
        e[1] = inv_dcc;
        e[2] = area;
        e[3] = kf;
      } else if (!same_geo(e[0], dcf) || !same_geo(e[1], inv_dcc) || !same_geo(e[2], area) || !same_geo(e[3], kf)) {
        snprintf(why, whylen, "the mixed path needs octree-regular geometry (cell %lld face %d)", (long long)c, f);
        return FVGPU_ERR_UNSUPPORTED;
      }
      // one area per level and axis for the single-neighbour faces (the
      // residual sums A (F- - F+) per axis)
      if (rel != kRelFiner) {
        const int ai = lev * 3 + axis_of_face(f);
        if (!seen_axis[ai]) {
          seen_axis[ai] = 1;
          gt.axis_area[ai] = area;
        } else if (!same_geo(gt.axis_area[ai], area)) {
          snprintf(why, whylen, "the mixed path needs equal areas of a cell's single-neighbour faces on an axis "
                                "(cell %lld face %d)", (long long)c, f);
          return FVGPU_ERR_UNSUPPORTED;
        }
      }
    }
    geom[size_t(c)] = code;
  }
  // the shared slope of a cell on an axis takes k from its + face: the two
  // same-level faces of an axis have the same dist_cf and dist_cc
  for (int lev = 0; lev <= kMaxLevel; ++lev)
    for (int ax = 0; ax < 3; ++ax) {
      const int ip = geo_index(lev, plus_face(ax), kRelSame), im = geo_index(lev, minus_face(ax), kRelSame);
      if (!seen[ip] || !seen[im]) continue;
      const float *ep = gt.face + ip * kGeoStride, *em = gt.face + im * kGeoStride;
      if (ep[0] != em[0] || ep[1] != em[1] || ep[3] != em[3]) {
        snprintf(why, whylen, "the mixed path needs the same cell spacing on both sides of an axis (level %d)", lev);
        return FVGPU_ERR_UNSUPPORTED;
      }
    }
  std::vector<BlockDesc> bricks;
  for (int64_t i = 0; i < n; i += Brick8::N) {
    BlockDesc d;
    memset(&d, 0, sizeof d);
    d.start = int(i);
    d.count = Brick8::N;
    d.level = m->level[i];
    for (int f = 0; f < 6; ++f) d.side[f] = brick_side<Brick8>(m, i, f, is_block8);
    bricks.push_back(d);
  }
  cudaError_t e;
  if ((e = allow_smem_brick(ph.ischeme == 2, ph.ns == 1)) != cudaSuccess) {
    snprintf(why, whylen, "shared-memory opt-in of the brick kernel: %s", cudaGetErrorString(e));
    return FVGPU_ERR_CUDA;
  }
  r.wave = brick_wave(ph.ischeme == 2, ph.ns == 1);
  if ((e = alloc_slot(r, kBufGeom, sizeof(int32_t) * n)) != cudaSuccess ||
      (e = cudaMemcpy(r.buf[kBufGeom], geom.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = alloc_slot(r, kBufTables, sizeof(GeoTables))) != cudaSuccess ||
      (e = cudaMemcpy(r.buf[kBufTables], &gt, sizeof gt, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = alloc_slot(r, kBufBlocks, sizeof(BlockDesc) * bricks.size())) != cudaSuccess ||
      (e = cudaMemcpy(r.buf[kBufBlocks], bricks.data(), sizeof(BlockDesc) * bricks.size(), cudaMemcpyHostToDevice)) !=
          cudaSuccess ||
      (e = alloc_slot(r, kBufD1, sizeof(float) * kNeqMax * n)) != cudaSuccess ||
      (e = alloc_slot(r, kBufD2, sizeof(float) * kNeqMax * n)) != cudaSuccess ||
      (e = alloc_slot(r, kBufAlt, sizeof(double) * kNeqMax * n)) != cudaSuccess ||
      (e = alloc_slot(r, kBufSNf, sizeof(float) * kNeqMax * n)) != cudaSuccess ||
      (e = alloc_slot(r, kBufSNfAlt, sizeof(float) * kNeqMax * n)) != cudaSuccess ||
      (e = alloc_slot(r, kBufX1, sizeof(float) * kNeqMax * n)) != cudaSuccess ||
      (e = alloc_slot(r, kBufX2, sizeof(float) * kNeqMax * n)) != cudaSuccess ||
      (e = alloc_slot(r, kBufSG, ph.ns == 1 ? sizeof(float) * 9 * n : 16)) != cudaSuccess) {
    snprintf(why, whylen, "mixed-path allocation: %s", cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? FVGPU_ERR_NOMEM : FVGPU_ERR_CUDA;
  }
  r.n = n;
  r.model = ph.model;
  r.nbricks = int64_t(bricks.size());
  r.nbricks4 = 0;
  r.ngeneral = 0;
  r.ready = true;
  return FVGPU_OK;
}

void release_mixed(MixedResources &r) {
  if (r.family == 1) {
    amr::release_mixed(r);
    r.family = 0;
    return;
  }
  for (int i = 0; i < 11; ++i) {
    if (r.buf[i]) cudaFree(r.buf[i]);
    r.buf[i] = nullptr;
    r.bytes[i] = 0;
    r.cap[i] = 0;
  }
  r.ready = false;
  r.snf_valid = false;
  r.nbricks = r.nbricks4 = r.ngeneral = 0;
}

void reset_mixed(MixedResources &r) {
  r.ready = false;
  r.snf_valid = false;
  r.nbricks = r.nbricks4 = r.ngeneral = 0;
  r.n = 0;
}

double *mixed_alt_state(MixedResources &r) { return static_cast<double *>(r.buf[kBufAlt]); }

// both families keep the second FP64 state in kBufAlt and the FP32 copies in
// kBufSNf / kBufSNfAlt
void mixed_swap_state(MixedResources &r, void *&state) {
  void *t = state;
  state = r.buf[kBufAlt];
  r.buf[kBufAlt] = t;
  t = r.buf[kBufSNf];
  r.buf[kBufSNf] = r.buf[kBufSNfAlt];
  r.buf[kBufSNfAlt] = t;
}

cudaError_t mixed_refresh_f32(MixedResources &r, const double *S, int neq, LaunchMarks &marks, cudaStream_t st) {
  if (r.family == 1) return amr::mixed_refresh_f32(r, S, neq, marks, st);
  marks.mark(FVGPU_KIND_MIXED_AUX);
  k_state_to_f32<1><<<1024, 256, 0, st>>>(S, static_cast<float *>(r.buf[kBufSNf]), r.n, neq);
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) r.snf_valid = true;
  return e;
}

cudaError_t mixed_refresh_f32_lambda(MixedResources &r, const Phys &ph, const double *S, double *lambda,
                                     LaunchMarks &marks, cudaStream_t st) {
  if (r.family == 1) return amr::mixed_refresh_f32_lambda(r, ph, S, lambda, marks, st);
  marks.mark(FVGPU_KIND_MIXED_AUX);
  const unsigned blocks = unsigned(std::min<int64_t>((r.n + kBlock - 1) / kBlock, 152 * 8));
  const MixedConst mc = make_const(ph);
  k_state_to_f32_lambda<1><<<blocks, kBlock, 0, st>>>(mc, static_cast<const int32_t *>(r.buf[kBufGeom]),
                                                      static_cast<const GeoTables *>(r.buf[kBufTables]), S,
                                                      static_cast<float *>(r.buf[kBufSNf]), int(r.n), lambda);
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) r.snf_valid = true;
  return e;
}

namespace {

// Dynamic shared memory above the 48 KiB default needs a per-kernel opt-in
// (cudaFuncAttributeMaxDynamicSharedMemorySize); it is set before any launch
// or stream capture (allow_smem_brick).

// the brick kernel of a configuration and stage kind (input increment,
// last stage)
template <bool MUSCL, bool NS>
const void *brick_kernel(bool din, bool last) {
  return din ? (last ? reinterpret_cast<const void *>(k_mixed_brick<1, MUSCL, NS, Brick8, 1, 1>)
                     : reinterpret_cast<const void *>(k_mixed_brick<1, MUSCL, NS, Brick8, 1, 0>))
             : (last ? reinterpret_cast<const void *>(k_mixed_brick<1, MUSCL, NS, Brick8, 0, 1>)
                     : reinterpret_cast<const void *>(k_mixed_brick<1, MUSCL, NS, Brick8, 0, 0>));
}
const void *brick_kernel_rt(bool muscl, bool ns, bool din, bool last) {
  return muscl ? (ns ? brick_kernel<true, true>(din, last) : brick_kernel<true, false>(din, last))
               : (ns ? brick_kernel<false, true>(din, last) : brick_kernel<false, false>(din, last));
}

cudaError_t launch_brick(bool muscl, unsigned grid, const MixedConst &mc, const StageArgs &a, cudaStream_t st) {
  constexpr size_t smem = Brick8::template smem_bytes<kNeqMax>();
  const void *k = brick_kernel_rt(muscl, mc.ns == 1, a.Din != nullptr, a.last != 0);
  MixedConst mc_ = mc;
  StageArgs a_ = a;
  void *args[] = {&mc_, &a_};
  return cudaLaunchKernel(k, dim3(grid), dim3(Brick8::N), args, smem, st);
}

}  // namespace

cudaError_t allow_smem_brick(bool muscl, bool ns) {
  constexpr size_t bytes = Brick8::template smem_bytes<kNeqMax>();
  for (int d = 0; d < 2; ++d)
    for (int l = 0; l < 2; ++l) {
      const cudaError_t e = cudaFuncSetAttribute(brick_kernel_rt(muscl, ns, d, l),
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes));
      if (e != cudaSuccess) return e;
    }
  return cudaSuccess;
}

int brick_wave(bool muscl, bool ns) {
  constexpr size_t smem = Brick8::template smem_bytes<kNeqMax>();
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, brick_kernel_rt(muscl, ns, true, false), Brick8::N,
                                                    smem) != cudaSuccess)
    return 0;
  return sms * per_sm;
}

// One RK step from FP64 state `in` (and its FP32 copy) to `out`.
cudaError_t enqueue_step_mixed(MixedResources &r, const Phys &ph, const MeshView &m, int scheme, bool cfl_mode,
                               const double *in, double *out, double *dt, double *lambda, const double *cfl,
                               unsigned long long *err, LaunchMarks &marks, cudaStream_t st) {
  if (r.family == 1)
    return amr::enqueue_step_mixed(r, ph, m, scheme, cfl_mode, in, out, dt, lambda, cfl, err, marks, st);
  static const int kStages[4][3] = {{0, 0, 0}, {1, 0, 0}, {1, 4, 0}, {1, 2, 3}};
  const int nst = scheme == 1 ? 1 : (scheme == 2 ? 2 : 3);
  if (cfl_mode) {
    marks.mark(FVGPU_KIND_DT);
    launch_dt_from_lambda(lambda, lambda, cfl, dt, err, st);
  }
  float *D[2] = {static_cast<float *>(r.buf[kBufD1]), static_cast<float *>(r.buf[kBufD2])};
  float *X[2] = {static_cast<float *>(r.buf[kBufX1]), static_cast<float *>(r.buf[kBufX2])};
  const MixedConst mc = make_const(ph);
  for (int k = 0; k < nst; ++k) {
    StageArgs a = stage_args(r, m);
    a.blocks = static_cast<const BlockDesc *>(r.buf[kBufBlocks]);
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
    a.ahead = r.wave;
    a.lambda = (a.last && cfl_mode) ? lambda : nullptr;
    a.err = err;
    if (ph.ns == 1) {
      marks.mark(FVGPU_KIND_MIXED_AUX);
      k_mixed_grad<1><<<unsigned((m.n + kBlock - 1) / kBlock), kBlock, 0, st>>>(mc, a,
                                                                               static_cast<float *>(r.buf[kBufSG]));
      const cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
    marks.mark(FVGPU_KIND_MIXED_STAGE);
    cudaError_t e = launch_brick(ph.ischeme == 2, unsigned(r.nbricks), mc, a, st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace fv
