// C ABI of libfvgpu (include/fvgpu.h): context, resident mesh and state,
// the reference's RHS / RK calls, graph-captured time steps, reductions.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../host/fvframes.h"
#include "fv_adjoint.cuh"
#include "fv_flatten.cuh"
#include "fv_kernels.cuh"
#include "fv_mixed.cuh"
#include "fvgpu.h"

namespace {

thread_local std::string g_create_error;

struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;  // the size asked for last
  size_t cap = 0;    // the size allocated (kept across meshes, reused when large enough)
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = cap = 0;
  }
  cudaError_t alloc(size_t b) {
    if (b == 0) b = 16;
    if (p && b <= cap) {
      bytes = b;
      return cudaSuccess;
    }
    release();
    cudaError_t e = cudaMalloc(&p, b);
    if (e == cudaSuccess) bytes = cap = b;
    else p = nullptr;
    return e;
  }
  template <typename T>
  T *as() const { return static_cast<T *>(p); }
};

struct GraphKey {
  int scheme, cfl, precision;
  const void *state;  // the graph bakes in the state buffer (mixed steps alternate two)
  bool operator<(const GraphKey &o) const {
    if (scheme != o.scheme) return scheme < o.scheme;
    if (cfl != o.cfl) return cfl < o.cfl;
    if (precision != o.precision) return precision < o.precision;
    return state < o.state;
  }
};

// device scalars, one allocation
struct Scalars {
  double dt;
  double lambda;
  double lambda_tmp;
  double cfl;
  unsigned long long err;
  unsigned long long pad[3];
};

}  // namespace

struct fvgpu_ctx {
  fvgpu_config cfg{};
  int neq = 5;
  cudaStream_t stream = nullptr;
  fv::Phys ph{};
  // mesh
  int64_t n = 0, nhang = 0;
  bool has_mesh = false;
  DevBuf nbr, nbr_face, area, dcf, dcc, vol, hang_nbr, hang_area, level, inner;
  // device flattening (fvgpu_upload_leaves): work arrays and the host copies
  // of the tables, kept across meshes and reused when large enough
  DevBuf lv_level, lv_ijk, lv_keys, lv_off, lv_tiles, lv_scal;
  std::vector<int32_t> lv_h32;
  std::vector<double> lv_h64;
  // state and work arrays
  DevBuf S, SN, R, SF, SG;
  DevBuf scal;      // Scalars
  DevBuf partial;   // conservation partial sums
  Scalars *h_scal = nullptr;  // pinned mirror
  bool lambda_valid = false;
  bool has_inner = false;
  // mixed-precision path resources
  fv::MixedResources mixed;
  bool mixed_ok = false;
  std::string mixed_why;
  // adjoint work arrays (allocated by the first adjoint call)
  unsigned bc_mask = 0;  // bit b set when boundary code b occurs in the mesh
  uint64_t mesh_sig = 0;  // FNV-1a of the uploaded tables (restart files carry it)
  bool mesh_sig_valid = false;  // formed on first use from the resident tables
  bool mesh_has_level = false;  // the upload carried per-cell levels
  DevBuf adjL, adjR, adjRh, adjW, adjG, adjAcc, adjOut, adjY1, adjY2, adjSN, adjCK;
  DevBuf adjGo, adjRg, adjRgh;  // viscous: gradient bars
  // halo exchange index lists
  DevBuf halo_send, halo_recv;
  int64_t nsend = 0, nrecv = 0;
  int64_t adj_ck_steps = 0;
  bool adj_ready = false;
  fv::LaunchMarks marks;
  std::map<GraphKey, cudaGraphExec_t> graphs;
  std::map<GraphKey, int> graph_launches;  // kernels per captured step
  // last error
  int last_code = 0;
  int64_t last_cell = -1;
  std::string last_msg;

  fv::MeshView view() const {
    fv::MeshView m;
    m.n = n;
    m.nhang = nhang;
    m.nbr = nbr.as<int32_t>();
    m.nbr_face = nbr_face.as<int32_t>();
    m.area = area.as<double>();
    m.dcf = dcf.as<double>();
    m.dcc = dcc.as<double>();
    m.vol = vol.as<double>();
    m.hang_nbr = hang_nbr.as<int32_t>();
    m.hang_area = hang_area.as<double>();
    return m;
  }
  Scalars *d_scal() const { return scal.as<Scalars>(); }
  double *d_dt() const { return &d_scal()->dt; }
  double *d_lambda() const { return &d_scal()->lambda; }
  double *d_lambda_tmp() const { return &d_scal()->lambda_tmp; }
  unsigned long long *d_err() const { return &d_scal()->err; }

  void drop_graphs() {
    for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
  }
};

namespace {

// FNV-1a, 64 bit
uint64_t fnv1a(uint64_t h, const void *data, size_t bytes) {
  const unsigned char *p = static_cast<const unsigned char *>(data);
  for (size_t i = 0; i < bytes; ++i) {
    h ^= p[i];
    h *= 0x100000001b3ull;
  }
  return h;
}
constexpr uint64_t kFnvSeed = 0xcbf29ce484222325ull;

// Face frames of an axis-aligned box, the same as fvmesh_flatten's
// (normalvector.c / tagvector.c; ../host/fvframes.h)
struct BoxFrames {
  double v[54];
  BoxFrames() { fv_box_frames(v); }
};
const BoxFrames kBoxFrames;

int set_err(fvgpu_ctx *ctx, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (ctx) {
    ctx->last_code = code;
    ctx->last_cell = -1;
    ctx->last_msg = buf;
  } else {
    g_create_error = buf;
  }
  return code;
}

#define FV_CUDA(ctx, call)                                                                   \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess)                                                                   \
      return set_err(ctx, e_ == cudaErrorMemoryAllocation ? FVGPU_ERR_NOMEM : FVGPU_ERR_CUDA, \
                     "%s: %s", #call, cudaGetErrorString(e_));                               \
  } while (0)

#define FV_LAUNCHED(ctx) FV_CUDA(ctx, cudaGetLastError())

// Conservation: fixed partition of the cells over kConsBlocks blocks, fixed
// in-block tree, fixed final tree -> the same sums on every run.
constexpr int kConsBlocks = 1024;
constexpr int kConsThreads = 256;

__global__ void k_cons_partial(int neq, int64_t n, const double *__restrict__ S, const double *__restrict__ vol,
                               double *__restrict__ partial) {
  __shared__ double red[kConsThreads];
  const int64_t per = (n + kConsBlocks - 1) / kConsBlocks;
  const int64_t lo = int64_t(blockIdx.x) * per;
  const int64_t hi = lo + per < n ? lo + per : n;
  for (int v = 0; v <= neq; ++v) {
    double acc = 0.0;
    for (int64_t c = lo + threadIdx.x; c < hi; c += kConsThreads)
      acc += v < neq ? S[v * n + c] * vol[c] : vol[c];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = kConsThreads / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0) partial[v * kConsBlocks + blockIdx.x] = red[0];
    __syncthreads();
  }
}

__global__ void k_cons_final(int neq, const double *__restrict__ partial, double *__restrict__ sums) {
  __shared__ double red[kConsThreads];
  for (int v = 0; v <= neq; ++v) {
    double acc = 0.0;
    for (int b = threadIdx.x; b < kConsBlocks; b += kConsThreads) acc += partial[v * kConsBlocks + b];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = kConsThreads / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0) sums[v] = red[0];
    __syncthreads();
  }
}

// refinement flags, criterionsplt.c:24-86 (pow(x, 2.0) is x*x in the
// compiled reference)
__global__ void k_criterion(int kind, double threshold, int level_hi, int64_t n, const double *__restrict__ S,
                            const double *__restrict__ SG, const double *__restrict__ vol, int32_t *__restrict__ split) {
  for (int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; c < n; c += int64_t(gridDim.x) * blockDim.x) {
    bool hit;
    if (kind == FVGPU_CRIT_RHO_BELOW) {
      hit = S[c] < threshold;
    } else {
      const double gx = SG[0 * n + c], gy = SG[1 * n + c], gz = SG[2 * n + c];
      // ((gx gx + gy gy) + gz gz) without contraction, as the reference evaluates it
      double mag = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(gx, gx), __dmul_rn(gy, gy)), __dmul_rn(gz, gz)));
      if (kind == FVGPU_CRIT_GRAD_RHO_H) mag = __dmul_rn(mag, cbrt(vol[c]));
      hit = mag > threshold;
    }
    split[c] = hit ? level_hi : 1;
  }
}

// halo exchange: gather / scatter of the state's rows
__global__ void k_halo_gather(int neq, int64_t n, const double *__restrict__ S, const int32_t *__restrict__ cells,
                              int64_t count, double *__restrict__ buf) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t c = cells[i];
    for (int v = 0; v < neq; ++v) buf[v * count + i] = S[v * n + c];
  }
}

__global__ void k_halo_scatter(int neq, int64_t n, double *__restrict__ S, const int32_t *__restrict__ cells,
                               int64_t count, const double *__restrict__ buf) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t c = cells[i];
    for (int v = 0; v < neq; ++v) S[v * n + c] = buf[v * count + i];
  }
}

__global__ void k_dt(const double *lambda_in, double *lambda_reset, const double *cflp, double *dt,
                     unsigned long long *err) {
  const double lam = *lambda_in;
  const double cfl = *cflp;
  if (!(lam > 0.0) || isinf(lam) || isnan(lam)) {
    *dt = 0.0;
    if (err && *err == 0ull) *err = (fv::kErrNonFinite << 40) | 0xffffffffffull;
  } else {
    *dt = cfl / lam;
  }
  if (lambda_reset) *lambda_reset = 0.0;
}

__global__ void k_set_double(double *p, double v) { *p = v; }

int check_device_error(fvgpu_ctx *ctx) {
  FV_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  const unsigned long long e = ctx->h_scal->err;
  if (e != 0ull) {
    const int code = int(e >> 40);
    const int64_t cell = int64_t(e & 0xffffffffffull);
    const int rc = code == int(fv::kErrEos) ? FVGPU_ERR_EOS : FVGPU_ERR_NONFINITE;
    set_err(ctx, rc, "device error %d at cell %lld (%s)", code, (long long)cell,
            code == 1 ? "non-finite residual or time step" : code == 2 ? "EOS without a real root"
                                                                       : "HLLC wave speeds not finite");
    ctx->last_cell = cell == 0xffffffffffll ? -1 : cell;
    // clear so the context stays usable
    ctx->h_scal->err = 0ull;
    FV_CUDA(ctx, cudaMemcpyAsync(ctx->d_err(), &ctx->h_scal->err, sizeof(unsigned long long),
                                 cudaMemcpyHostToDevice, ctx->stream));
    FV_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return rc;
  }
  return FVGPU_OK;
}

// Pull the device error word into the pinned mirror (async) and check.
int sync_and_check(fvgpu_ctx *ctx) {
  FV_CUDA(ctx, cudaMemcpyAsync(&ctx->h_scal->err, ctx->d_err(), sizeof(unsigned long long),
                               cudaMemcpyDeviceToHost, ctx->stream));
  return check_device_error(ctx);
}

int validate_config(const fvgpu_config *c, char *why, size_t whylen) {
  if (c->model < 1 || c->model > 3) {
    snprintf(why, whylen,
             "model %d unsupported (1-3; the reference's model 4 accumulates no flux, "
             "residual_faces_AMR.c:216-236)",
             c->model);
    return FVGPU_ERR_UNSUPPORTED;
  }
  if (c->iprimtv != 0) {
    snprintf(why, whylen,
             "iprimtv=1 unsupported: the reference's cons2primtv reads sol->r, which "
             "facevalues_MUSCL never sets (cons2primtv.c:5, facevalues_MUSCL.c:3-56)");
    return FVGPU_ERR_UNSUPPORTED;
  }
  if (c->ischeme != 1 && c->ischeme != 2) {
    snprintf(why, whylen, "ischeme must be 1 or 2");
    return FVGPU_ERR_ARG;
  }
  if (c->ns != 0 && c->ns != 1) {
    snprintf(why, whylen, "ns must be 0 or 1");
    return FVGPU_ERR_ARG;
  }
  if (c->precision != FVGPU_FP64 && c->precision != FVGPU_MIXED) {
    snprintf(why, whylen, "precision must be FVGPU_FP64 or FVGPU_MIXED");
    return FVGPU_ERR_ARG;
  }
  if (c->model == 1 && !(c->gamma > 1.0)) {
    snprintf(why, whylen, "gamma must exceed 1");
    return FVGPU_ERR_ARG;
  }
  return FVGPU_OK;
}

fv::Phys make_phys(const fvgpu_config &c, int neq, const double *frames) {
  fv::Phys p{};
  p.model = c.model;
  p.ns = c.ns;
  p.ischeme = c.ischeme;
  p.eos = c.eos;
  p.neq = neq;
  p.gamma = c.gamma;
  p.pinf = c.pinf;
  p.visc = c.visc;
  p.ymin = c.ymin;
  for (int i = 0; i < 8; ++i) p.inflow[i] = c.inflow[i];
  if (frames)
    for (int i = 0; i < 54; ++i) p.frames[i] = frames[i];
  return p;
}

// Host-side validation of the flattened tables: every index in range,
// geometry positive and finite, and each face link reciprocated by the
// neighbour's face (1:1, coarse-to-fine and fine-to-coarse).
int validate_mesh(fvgpu_ctx *ctx, const fvgpu_mesh_soa *m) {
  const int64_t n = m->ncells, nh = m->nhang;
  if (n <= 0 || n >= (int64_t(1) << 31)) return set_err(ctx, FVGPU_ERR_MESH, "ncells %lld out of range", (long long)n);
  if (nh < 0 || nh > 6 * n) return set_err(ctx, FVGPU_ERR_MESH, "nhang %lld out of range", (long long)nh);
  if (!m->nbr || !m->nbr_face || !m->area || !m->dcf || !m->dcc || !m->vol || !m->frames ||
      (nh > 0 && (!m->hang_nbr || !m->hang_area)))
    return set_err(ctx, FVGPU_ERR_ARG, "null mesh array");
  for (int i = 0; i < 54; ++i)
    if (!std::isfinite(m->frames[i])) return set_err(ctx, FVGPU_ERR_MESH, "non-finite face frame");
  for (int64_t c = 0; c < n; ++c)
    if (!(m->vol[c] > 0.0) || !std::isfinite(m->vol[c]))
      return set_err(ctx, FVGPU_ERR_MESH, "cell %lld: volume must be positive", (long long)c);
  std::vector<uint8_t> hang_seen(size_t(nh), 0);
  for (int f = 0; f < 6; ++f) {
    for (int64_t c = 0; c < n; ++c) {
      const int64_t i = f * n + c;
      const int32_t code = m->nbr[i];
      const double A = m->area[i], dcf = m->dcf[i], dcc = m->dcc[i];
      if (!(dcf >= 0.0) || !(dcc >= 0.0) || !std::isfinite(dcf) || !std::isfinite(dcc))
        return set_err(ctx, FVGPU_ERR_MESH, "cell %lld face %d: bad stencil distance", (long long)c, f);
      if (code < 0 && code > FVGPU_HANG0) {
        const int bc = -1 - code;
        if (bc < 1 || bc > 4)
          return set_err(ctx, FVGPU_ERR_MESH, "cell %lld face %d: boundary code %d not in 1..4", (long long)c, f, bc);
        if (bc == 1 && ctx->cfg.model != 1)
          return set_err(ctx, FVGPU_ERR_UNSUPPORTED,
                         "inflow boundaries need model 1 (asinvalues_multiphase.c:22 fills the other side)");
        if (!(A > 0.0) || !std::isfinite(A))
          return set_err(ctx, FVGPU_ERR_MESH, "cell %lld face %d: area must be positive", (long long)c, f);
        continue;
      }
      const int nf = m->nbr_face[i];
      if (nf < 0 || nf > 5)
        return set_err(ctx, FVGPU_ERR_MESH, "cell %lld face %d: neighbour face %d", (long long)c, f, nf);
      if (!(dcc > 0.0))
        return set_err(ctx, FVGPU_ERR_MESH, "cell %lld face %d: interior face needs dcc > 0", (long long)c, f);
      if (code >= 0) {
        if (code >= n) return set_err(ctx, FVGPU_ERR_MESH, "cell %lld face %d: neighbour %d out of range", (long long)c, f, code);
        if (!(A > 0.0) || !std::isfinite(A))
          return set_err(ctx, FVGPU_ERR_MESH, "cell %lld face %d: area must be positive", (long long)c, f);
        // reciprocity: neighbour's face nf points back at c, or is a 1:4 face containing c
        const int32_t back = m->nbr[int64_t(nf) * n + code];
        bool ok = back == c;
        if (!ok && back <= FVGPU_HANG0) {
          const int64_t r = int64_t(FVGPU_HANG0) - back;
          if (r < nh)
            for (int s = 0; s < 4; ++s) ok |= m->hang_nbr[4 * r + s] == c;
        }
        if (!ok)
          return set_err(ctx, FVGPU_ERR_MESH, "cell %lld face %d: neighbour %d does not link back", (long long)c, f, code);
      } else {
        const int64_t r = int64_t(FVGPU_HANG0) - code;
        if (r >= nh) return set_err(ctx, FVGPU_ERR_MESH, "cell %lld face %d: hanging record %lld out of range", (long long)c, f, (long long)r);
        if (hang_seen[size_t(r)]) return set_err(ctx, FVGPU_ERR_MESH, "hanging record %lld used twice", (long long)r);
        hang_seen[size_t(r)] = 1;
        for (int s = 0; s < 4; ++s) {
          const int32_t k = m->hang_nbr[4 * r + s];
          const double a = m->hang_area[4 * r + s];
          if (k < 0 || k >= n) return set_err(ctx, FVGPU_ERR_MESH, "hanging record %lld: neighbour out of range", (long long)r);
          if (!(a > 0.0) || !std::isfinite(a)) return set_err(ctx, FVGPU_ERR_MESH, "hanging record %lld: area must be positive", (long long)r);
          if (m->nbr[int64_t(nf) * n + k] != c)
            return set_err(ctx, FVGPU_ERR_MESH, "hanging record %lld: fine neighbour %d does not link back", (long long)r, k);
        }
      }
    }
  }
  return FVGPU_OK;
}

int ensure_state(fvgpu_ctx *ctx) {
  if (!ctx) return FVGPU_ERR_ARG;
  if (!ctx->has_mesh) return set_err(ctx, FVGPU_ERR_STATE, "no mesh uploaded");
  return FVGPU_OK;
}

// ---- launch sequences -------------------------------------------------------

int enqueue_faceinterp(fvgpu_ctx *ctx) {
  ctx->marks.mark(FVGPU_KIND_FACEINTERP);
  fv::launch_faceinterp_fp64(ctx->ph, ctx->view(), ctx->S.as<double>(), ctx->SF.as<double>(), ctx->stream);
  FV_LAUNCHED(ctx);
  return FVGPU_OK;
}

int enqueue_gradcalc(fvgpu_ctx *ctx) {
  ctx->marks.mark(FVGPU_KIND_GRADCALC);
  fv::launch_gradcalc_fp64(ctx->ph, ctx->view(), ctx->S.as<double>(), ctx->SG.as<double>(), ctx->d_err(),
                           ctx->stream);
  FV_LAUNCHED(ctx);
  return FVGPU_OK;
}

fv::ResidualArgs residual_args(fvgpu_ctx *ctx) {
  fv::ResidualArgs a{};
  a.U = ctx->S.as<double>();
  a.SF = ctx->SF.as<double>();
  a.SG = ctx->SG.as<double>();
  a.R = ctx->R.as<double>();
  a.S_out = ctx->S.as<double>();
  a.SN = ctx->SN.as<double>();
  a.dt = ctx->d_dt();
  a.lambda = nullptr;
  a.inner = nullptr;
  a.inner_outer = 0;
  a.irk = 0;
  a.err = ctx->d_err();
  return a;
}

int enqueue_rhs(fvgpu_ctx *ctx, const int32_t *inner, int inner_outer) {
  fv::ResidualArgs a = residual_args(ctx);
  a.inner = inner;
  a.inner_outer = inner_outer;
  ctx->marks.mark(FVGPU_KIND_RESIDUAL);
  fv::launch_residual_fp64(ctx->ph, ctx->view(), a, ctx->stream);
  FV_LAUNCHED(ctx);
  return FVGPU_OK;
}

// One RK step: stages of `scheme`; CFL dt from lambda when cfl_mode.
int enqueue_step_fp64(fvgpu_ctx *ctx, int scheme, bool cfl_mode) {
  static const int kStages[4][3] = {{0, 0, 0}, {1, 0, 0}, {1, 4, 0}, {1, 2, 3}};
  static const int kN[4] = {0, 1, 2, 3};
  if (cfl_mode) {
    ctx->marks.mark(FVGPU_KIND_DT);
    k_dt<<<1, 1, 0, ctx->stream>>>(ctx->d_lambda(), ctx->d_lambda(), &ctx->d_scal()->cfl, ctx->d_dt(),
                                   ctx->d_err());
    FV_LAUNCHED(ctx);
  }
  const int ns = kN[scheme];
  const fv::MeshView mv = ctx->view();
  if (ctx->cfg.ischeme == 1) {
    ctx->marks.mark(FVGPU_KIND_RK);
    fv::launch_rk_fp64(0, ctx->ph, mv, ctx->S.as<double>(), ctx->SN.as<double>(), ctx->R.as<double>(),
                       ctx->d_dt(), nullptr, ctx->stream);
    FV_LAUNCHED(ctx);
  }
  for (int k = 0; k < ns; ++k) {
    const int irk = kStages[scheme][k];
    const bool last = k == ns - 1;
    if (ctx->cfg.ischeme == 2) {
      int rc = enqueue_faceinterp(ctx);
      if (rc) return rc;
    }
    if (ctx->cfg.ns == 1) {
      int rc = enqueue_gradcalc(ctx);
      if (rc) return rc;
    }
    if (ctx->cfg.ischeme == 2) {
      fv::ResidualArgs a = residual_args(ctx);
      a.R = nullptr;
      a.irk = irk;
      a.lambda = (last && cfl_mode) ? ctx->d_lambda() : nullptr;
      ctx->marks.mark(FVGPU_KIND_RESIDUAL);
      fv::launch_residual_fp64(ctx->ph, mv, a, ctx->stream);
      FV_LAUNCHED(ctx);
    } else {
      int rc = enqueue_rhs(ctx, nullptr, 0);
      if (rc) return rc;
      ctx->marks.mark(FVGPU_KIND_RK);
      fv::launch_rk_fp64(irk, ctx->ph, mv, ctx->S.as<double>(), ctx->SN.as<double>(), ctx->R.as<double>(),
                         ctx->d_dt(), (last && cfl_mode) ? ctx->d_lambda() : nullptr, ctx->stream);
      FV_LAUNCHED(ctx);
    }
  }
  return FVGPU_OK;
}

int enqueue_step(fvgpu_ctx *ctx, int scheme, bool cfl_mode) {
  if (ctx->cfg.precision == FVGPU_MIXED) {
    const cudaError_t e = fv::enqueue_step_mixed(ctx->mixed, ctx->ph, ctx->view(), scheme, cfl_mode,
                                                 ctx->S.as<double>(), fv::mixed_alt_state(ctx->mixed), ctx->d_dt(),
                                                 ctx->d_lambda(), &ctx->d_scal()->cfl, ctx->d_err(), ctx->marks,
                                                 ctx->stream);
    return e == cudaSuccess ? FVGPU_OK : set_err(ctx, FVGPU_ERR_CUDA, "mixed step launch: %s", cudaGetErrorString(e));
  }
  return enqueue_step_fp64(ctx, scheme, cfl_mode);
}

// after a step has been queued: the mixed path wrote the new state into the
// second buffer, which becomes the current state
void after_step(fvgpu_ctx *ctx) {
  if (ctx->cfg.precision == FVGPU_MIXED)
    fv::mixed_swap_state(ctx->mixed, ctx->S.p);
  else
    ctx->mixed.snf_valid = false;
}

// the mixed path reads an FP32 copy of the state; rebuild it when the state
// changed outside a mixed step
int ensure_mixed_f32(fvgpu_ctx *ctx) {
  if (ctx->cfg.precision != FVGPU_MIXED || ctx->mixed.snf_valid) return FVGPU_OK;
  const cudaError_t e = fv::mixed_refresh_f32(ctx->mixed, ctx->S.as<double>(), ctx->neq, ctx->marks, ctx->stream);
  return e == cudaSuccess ? FVGPU_OK : set_err(ctx, FVGPU_ERR_CUDA, "state copy: %s", cudaGetErrorString(e));
}

int ensure_lambda(fvgpu_ctx *ctx) {
  if (ctx->lambda_valid) return FVGPU_OK;
  FV_CUDA(ctx, cudaMemsetAsync(ctx->d_lambda(), 0, sizeof(double), ctx->stream));
  if (ctx->cfg.precision == FVGPU_MIXED) {
    // the mixed path's radius is FP32 (as at the end of its steps); one pass
    // also rebuilds the FP32 copy of the state
    const cudaError_t e = fv::mixed_refresh_f32_lambda(ctx->mixed, ctx->ph, ctx->S.as<double>(), ctx->d_lambda(),
                                                       ctx->marks, ctx->stream);
    if (e != cudaSuccess) return set_err(ctx, FVGPU_ERR_CUDA, "state copy: %s", cudaGetErrorString(e));
    ctx->lambda_valid = true;
    return FVGPU_OK;
  }
  ctx->marks.mark(FVGPU_KIND_DT);
  fv::launch_lambda_fp64(ctx->ph, ctx->view(), ctx->S.as<double>(), ctx->d_lambda(), ctx->stream);
  FV_LAUNCHED(ctx);
  ctx->lambda_valid = true;
  return FVGPU_OK;
}

// ---- adjoint ---------------------------------------------------------------

int ensure_adjoint(fvgpu_ctx *ctx) {
  char why[256] = {0};
  if (!fv::adjoint_supported(ctx->ph, why, sizeof why)) return set_err(ctx, FVGPU_ERR_UNSUPPORTED, "%s", why);
  if (ctx->bc_mask & ((1u << 3) | (1u << 4)))
    return set_err(ctx, FVGPU_ERR_UNSUPPORTED, "the adjoint does not implement the wall boundary codes 3 and 4");
  if (ctx->adj_ready) return FVGPU_OK;
  const size_t cell = sizeof(double) * size_t(ctx->neq) * size_t(ctx->n);
  FV_CUDA(ctx, ctx->adjL.alloc(6 * cell));
  FV_CUDA(ctx, ctx->adjR.alloc(6 * cell));
  FV_CUDA(ctx, ctx->adjRh.alloc(sizeof(double) * 4 * size_t(ctx->neq) * size_t(ctx->nhang)));
  for (DevBuf *b : {&ctx->adjW, &ctx->adjG, &ctx->adjAcc, &ctx->adjOut, &ctx->adjY1, &ctx->adjY2, &ctx->adjSN})
    FV_CUDA(ctx, b->alloc(cell));
  if (ctx->cfg.ns == 1) {
    const size_t row = sizeof(double) * size_t(ctx->n);
    FV_CUDA(ctx, ctx->adjGo.alloc(9 * row));
    FV_CUDA(ctx, ctx->adjRg.alloc(54 * row));
    FV_CUDA(ctx, ctx->adjRgh.alloc(sizeof(double) * 36 * size_t(ctx->nhang)));
  }
  ctx->adj_ready = true;
  return FVGPU_OK;
}

// out = (dR/dU)^T w at U (all device arrays [neq][n]) with the reverse
// passes in FP32: face values, fluxes, limiter and EOS reversed in FP32, the
// intermediate arrays FP32 (in the FP64 buffers), FP64 gradients for the
// viscous flux; overwrites SF
int enqueue_vjp_f32(fvgpu_ctx *ctx, const double *U, const double *w, double *out) {
  const fv::MeshView mv = ctx->view();
  if (ctx->cfg.ischeme == 2) {
    ctx->marks.mark(FVGPU_KIND_FACEINTERP);
    fv::launch_faceinterp_f32(ctx->ph, mv, U, ctx->SF.as<float>(), ctx->stream);
    FV_LAUNCHED(ctx);
  }
  if (ctx->cfg.ns == 1) {
    ctx->marks.mark(FVGPU_KIND_GRADCALC);
    fv::launch_gradcalc_fp64(ctx->ph, mv, U, ctx->SG.as<double>(), ctx->d_err(), ctx->stream);
    FV_LAUNCHED(ctx);
  }
  fv::AdjArgsT<float> a{};
  a.U = U;
  a.SF = ctx->SF.as<float>();
  a.w = w;
  a.gL = ctx->adjL.as<float>();
  a.gR = ctx->adjR.as<float>();
  a.gRh = ctx->adjRh.as<float>();
  a.gSF = ctx->adjL.as<float>();
  a.out = out;
  a.SG = ctx->SG.as<double>();
  a.gG = ctx->adjGo.as<float>();
  a.gRg = ctx->adjRg.as<float>();
  a.gRgh = ctx->adjRgh.as<float>();
  a.gSG = ctx->adjGo.as<float>();
  ctx->marks.mark(FVGPU_KIND_ADJOINT);
  fv::launch_adjoint_f32(ctx->ph, mv, a, ctx->stream);
  FV_LAUNCHED(ctx);
  return FVGPU_OK;
}

// out = (dR/dU)^T w at U (all device arrays [neq][n]); overwrites SF.  A
// context on the FP32-mixed path runs the FP32 reverse passes.
int enqueue_vjp(fvgpu_ctx *ctx, const double *U, const double *w, double *out) {
  if (ctx->cfg.precision == FVGPU_MIXED) return enqueue_vjp_f32(ctx, U, w, out);
  const fv::MeshView mv = ctx->view();
  if (ctx->cfg.ischeme == 2) {
    ctx->marks.mark(FVGPU_KIND_FACEINTERP);
    fv::launch_faceinterp_fp64(ctx->ph, mv, U, ctx->SF.as<double>(), ctx->stream);
    FV_LAUNCHED(ctx);
  }
  if (ctx->cfg.ns == 1) {
    ctx->marks.mark(FVGPU_KIND_GRADCALC);
    fv::launch_gradcalc_fp64(ctx->ph, mv, U, ctx->SG.as<double>(), ctx->d_err(), ctx->stream);
    FV_LAUNCHED(ctx);
  }
  fv::AdjArgs a{};
  a.U = U;
  a.SF = ctx->SF.as<double>();
  a.w = w;
  a.gL = ctx->adjL.as<double>();
  a.gR = ctx->adjR.as<double>();
  a.gRh = ctx->adjRh.as<double>();
  a.gSF = ctx->adjL.as<double>();  // each face's total replaces its own-evaluation part in place
  a.out = out;
  a.SG = ctx->SG.as<double>();
  a.gG = ctx->adjGo.as<double>();
  a.gRg = ctx->adjRg.as<double>();
  a.gRgh = ctx->adjRgh.as<double>();
  a.gSG = ctx->adjGo.as<double>();  // likewise for the gradient bars
  ctx->marks.mark(FVGPU_KIND_ADJOINT);
  fv::launch_adjoint(ctx->ph, mv, a, ctx->stream);
  FV_LAUNCHED(ctx);
  return FVGPU_OK;
}

// RK stage coefficients: S_out = a SN + b S_in + b dt / V R(S_in) (RK.c:16-47)
void stage_coef(int irk, double &a, double &b) {
  switch (irk) {
    case 2: a = 3.0 / 4.0; b = 1.0 / 4.0; break;
    case 3: a = 1.0 / 3.0; b = 2.0 / 3.0; break;
    case 4: a = 1.0 / 2.0; b = 1.0 / 2.0; break;
    default: a = 0.0; b = 1.0; break;
  }
}

const int kSchemeStages[4][3] = {{0, 0, 0}, {1, 0, 0}, {1, 4, 0}, {1, 2, 3}};

// forward stage irk from S_in into S_out (out of place), SN in ctx->adjSN
int enqueue_stage_out_of_place(fvgpu_ctx *ctx, int irk, const double *S_in, double *S_out) {
  if (ctx->cfg.ischeme == 2) {
    ctx->marks.mark(FVGPU_KIND_FACEINTERP);
    fv::launch_faceinterp_fp64(ctx->ph, ctx->view(), S_in, ctx->SF.as<double>(), ctx->stream);
    FV_LAUNCHED(ctx);
  }
  if (ctx->cfg.ns == 1) {
    ctx->marks.mark(FVGPU_KIND_GRADCALC);
    fv::launch_gradcalc_fp64(ctx->ph, ctx->view(), S_in, ctx->SG.as<double>(), ctx->d_err(), ctx->stream);
    FV_LAUNCHED(ctx);
  }
  fv::ResidualArgs a = residual_args(ctx);
  a.U = S_in;
  a.R = nullptr;
  a.S_out = S_out;
  a.SN = ctx->adjSN.as<double>();
  a.irk = irk;
  ctx->marks.mark(FVGPU_KIND_RESIDUAL);
  fv::launch_residual_fp64(ctx->ph, ctx->view(), a, ctx->stream);
  FV_LAUNCHED(ctx);
  return FVGPU_OK;
}

// G <- (dS_out/dS_in)^T G for one step from the checkpoint X0 (device, [neq][n])
int enqueue_step_adjoint(fvgpu_ctx *ctx, int scheme, const double *X0) {
  const int ns = scheme;  // stages per step: 1, 2, 3
  const int64_t count = int64_t(ctx->neq) * ctx->n;
  const double *X[3] = {X0, ctx->adjY1.as<double>(), ctx->adjY2.as<double>()};
  double *G = ctx->adjG.as<double>(), *Acc = ctx->adjAcc.as<double>();
  for (int j = 0; j + 1 < ns; ++j) {
    int rc = enqueue_stage_out_of_place(ctx, kSchemeStages[scheme][j], X[j], const_cast<double *>(X[j + 1]));
    if (rc) return rc;
  }
  FV_CUDA(ctx, cudaMemsetAsync(Acc, 0, sizeof(double) * size_t(count), ctx->stream));
  for (int j = ns - 1; j >= 0; --j) {
    double a, b;
    stage_coef(kSchemeStages[scheme][j], a, b);
    if (a != 0.0) {
      fv::launch_axpby(count, a, G, 1.0, Acc, ctx->stream);
      FV_LAUNCHED(ctx);
    }
    fv::launch_adj_scale(ctx->view(), G, ctx->d_dt(), b, ctx->adjW.as<double>(), ctx->stream);
    FV_LAUNCHED(ctx);
    int rc = enqueue_vjp(ctx, X[j], ctx->adjW.as<double>(), ctx->adjOut.as<double>());
    if (rc) return rc;
    fv::launch_axpby(count, 1.0, ctx->adjOut.as<double>(), b, G, ctx->stream);
    FV_LAUNCHED(ctx);
  }
  fv::launch_axpby(count, 1.0, Acc, 1.0, G, ctx->stream);
  FV_LAUNCHED(ctx);
  return FVGPU_OK;
}

}  // namespace

namespace fv {
void launch_dt_from_lambda(const double *lambda_in, double *lambda_reset, const double *cfl, double *dt,
                           unsigned long long *err, cudaStream_t st) {
  k_dt<<<1, 1, 0, st>>>(lambda_in, lambda_reset, cfl, dt, err);
}
}  // namespace fv

extern "C" {

int fvgpu_create(const fvgpu_config *cfg, fvgpu_ctx **out) {
  if (!cfg || !out) return set_err(nullptr, FVGPU_ERR_ARG, "null argument");
  *out = nullptr;
  char why[256];
  int rc = validate_config(cfg, why, sizeof why);
  if (rc) return set_err(nullptr, rc, "%s", why);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return set_err(nullptr, FVGPU_ERR_NODEVICE, "no CUDA device");
  }
  if (cfg->device < 0 || cfg->device >= ndev) return set_err(nullptr, FVGPU_ERR_ARG, "device %d out of range", cfg->device);
  if (cudaSetDevice(cfg->device) != cudaSuccess) return set_err(nullptr, FVGPU_ERR_CUDA, "cudaSetDevice failed");
  fvgpu_ctx *ctx = new fvgpu_ctx();
  ctx->cfg = *cfg;
  ctx->neq = cfg->model == 2 ? 4 : 5;
  ctx->ph = make_phys(*cfg, ctx->neq, nullptr);
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
      ctx->scal.alloc(sizeof(Scalars)) != cudaSuccess ||
      cudaMallocHost((void **)&ctx->h_scal, sizeof(Scalars)) != cudaSuccess ||
      ctx->partial.alloc(sizeof(double) * (kConsBlocks * (fv::kNeqMax + 1) + 8)) != cudaSuccess) {
    cudaGetLastError();
    delete ctx;
    return set_err(nullptr, FVGPU_ERR_CUDA, "context allocation failed");
  }
  memset(ctx->h_scal, 0, sizeof(Scalars));
  if (cudaMemset(ctx->scal.p, 0, sizeof(Scalars)) != cudaSuccess) {
    delete ctx;
    return set_err(nullptr, FVGPU_ERR_CUDA, "cudaMemset failed");
  }
  *out = ctx;
  return FVGPU_OK;
}

int fvgpu_destroy(fvgpu_ctx *ctx) {
  if (!ctx) return FVGPU_OK;
  cudaSetDevice(ctx->cfg.device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  ctx->drop_graphs();
  fv::release_mixed(ctx->mixed);
  if (ctx->h_scal) cudaFreeHost(ctx->h_scal);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return FVGPU_OK;
}

int fvgpu_neq(const fvgpu_ctx *ctx) { return ctx ? ctx->neq : 0; }

int fvgpu_set_precision(fvgpu_ctx *ctx, int precision) {
  if (!ctx) return FVGPU_ERR_ARG;
  if (precision != FVGPU_FP64 && precision != FVGPU_MIXED)
    return set_err(ctx, FVGPU_ERR_ARG, "precision must be FVGPU_FP64 or FVGPU_MIXED");
  if (precision == ctx->cfg.precision) return FVGPU_OK;
  cudaSetDevice(ctx->cfg.device);
  if (precision == FVGPU_MIXED) {
    char why[256];
    if (!fv::mixed_supported(ctx->ph, why, sizeof why)) return set_err(ctx, FVGPU_ERR_UNSUPPORTED, "%s", why);
    if (ctx->has_mesh && !ctx->mixed_ok)
      return set_err(ctx, FVGPU_ERR_UNSUPPORTED, "%s", ctx->mixed_why.c_str());
  }
  ctx->cfg.precision = precision;
  ctx->mixed.snf_valid = false;
  ctx->drop_graphs();
  return FVGPU_OK;
}

static int finish_mesh(fvgpu_ctx *ctx, const fvgpu_mesh_soa *m);

int fvgpu_upload_mesh(fvgpu_ctx *ctx, const fvgpu_mesh_soa *m) {
  if (!ctx || !m) return set_err(ctx, FVGPU_ERR_ARG, "null argument");
  int rc = validate_mesh(ctx, m);
  if (rc) return rc;
  cudaSetDevice(ctx->cfg.device);
  FV_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->drop_graphs();
  fv::reset_mixed(ctx->mixed);
  ctx->has_mesh = false;
  const int64_t n = m->ncells, nh = m->nhang;
  const int neq = ctx->neq;
  struct Up {
    DevBuf *buf;
    const void *src;
    size_t bytes;
  } ups[] = {
      {&ctx->nbr, m->nbr, sizeof(int32_t) * 6 * n},     {&ctx->nbr_face, m->nbr_face, sizeof(int32_t) * 6 * n},
      {&ctx->area, m->area, sizeof(double) * 6 * n},    {&ctx->dcf, m->dcf, sizeof(double) * 6 * n},
      {&ctx->dcc, m->dcc, sizeof(double) * 6 * n},      {&ctx->vol, m->vol, sizeof(double) * n},
      {&ctx->hang_nbr, m->hang_nbr, sizeof(int32_t) * 4 * nh},
      {&ctx->hang_area, m->hang_area, sizeof(double) * 4 * nh},
      {&ctx->level, m->level, m->level ? sizeof(int32_t) * n : 0},
  };
  for (auto &u : ups) {
    FV_CUDA(ctx, u.buf->alloc(u.bytes));
    if (u.src && u.bytes) FV_CUDA(ctx, cudaMemcpy(u.buf->p, u.src, u.bytes, cudaMemcpyHostToDevice));
  }
  return finish_mesh(ctx, m);
}

// Everything after the tables are on the device: state and work arrays,
// mesh signature, boundary codes present, the mixed path's tables.  m holds
// host copies of the same tables.
static int finish_mesh(fvgpu_ctx *ctx, const fvgpu_mesh_soa *m) {
  const int64_t n = m->ncells, nh = m->nhang;
  const int neq = ctx->neq;
  FV_CUDA(ctx, ctx->S.alloc(sizeof(double) * neq * n));
  FV_CUDA(ctx, ctx->SN.alloc(sizeof(double) * neq * n));
  FV_CUDA(ctx, ctx->R.alloc(sizeof(double) * neq * n));
  FV_CUDA(ctx, ctx->SF.alloc(ctx->cfg.ischeme == 2 ? sizeof(double) * 6 * neq * n : 16));
  FV_CUDA(ctx, ctx->SG.alloc(ctx->cfg.ns == 1 ? sizeof(double) * (neq + 1) * 3 * n : 16));
  FV_CUDA(ctx, cudaMemset(ctx->S.p, 0, ctx->S.bytes));
  FV_CUDA(ctx, cudaMemset(ctx->SN.p, 0, ctx->SN.bytes));
  FV_CUDA(ctx, cudaMemset(ctx->R.p, 0, ctx->R.bytes));
  FV_CUDA(ctx, cudaMemset(ctx->SF.p, 0, ctx->SF.bytes));
  FV_CUDA(ctx, cudaMemset(ctx->SG.p, 0, ctx->SG.bytes));
  ctx->inner.release();
  ctx->has_inner = false;
  for (DevBuf *b : {&ctx->adjL, &ctx->adjR, &ctx->adjRh, &ctx->adjW, &ctx->adjG, &ctx->adjAcc, &ctx->adjOut,
                    &ctx->adjY1, &ctx->adjY2, &ctx->adjSN, &ctx->adjCK, &ctx->adjGo, &ctx->adjRg, &ctx->adjRgh})
    b->release();
  ctx->adj_ck_steps = 0;
  ctx->adj_ready = false;
  ctx->halo_send.release();
  ctx->halo_recv.release();
  ctx->nsend = ctx->nrecv = 0;
  // the signature is formed when a restart or a caller first asks for it
  ctx->mesh_sig_valid = false;
  ctx->mesh_has_level = m->level != nullptr;
  ctx->bc_mask = 0;
  for (int64_t i = 0; i < 6 * n; ++i) {
    const int32_t code = m->nbr[i];
    if (code < 0 && code > FVGPU_HANG0) ctx->bc_mask |= 1u << (-1 - code);
  }
  ctx->n = n;
  ctx->nhang = nh;
  ctx->ph = make_phys(ctx->cfg, neq, m->frames);
  ctx->lambda_valid = false;
  {
    char why[256] = {0};
    ctx->mixed.force_general = (ctx->cfg.flags & FVGPU_FLAG_NO_BRICKS) != 0;
    ctx->mixed_ok = fv::mixed_prepare_host(ctx->mixed, ctx->ph, m, why, sizeof why) == FVGPU_OK;
    ctx->mixed_why = why;
    if (ctx->cfg.precision == FVGPU_MIXED && !ctx->mixed_ok)
      return set_err(ctx, FVGPU_ERR_UNSUPPORTED, "%s", why);
  }
  FV_CUDA(ctx, cudaDeviceSynchronize());
  ctx->has_mesh = true;
  return FVGPU_OK;
}

int fvgpu_upload_leaves(fvgpu_ctx *ctx, const fvgpu_leaves *lv) {
  if (!ctx || !lv) return set_err(ctx, FVGPU_ERR_ARG, "null argument");
  const int64_t n = lv->ncells;
  if (n <= 0 || n > 300000000 || !lv->level || !lv->ijk)  // 6 n record numbers fit int32
    return set_err(ctx, FVGPU_ERR_ARG, "need 1 <= ncells <= 3e8 and level / ijk arrays");
  fv::LeafGeom g;
  for (int a = 0; a < 3; ++a) {
    g.lo[a] = lv->lo[a];
    g.len[a] = lv->len[a];
    g.periodic[a] = lv->periodic[a] ? 1 : 0;
    if (!(g.len[a] > 0.0) || !std::isfinite(g.lo[a])) return set_err(ctx, FVGPU_ERR_ARG, "bad box");
  }
  static const int kAxisOf[6] = {1, 0, 1, 0, 2, 2};
  for (int f = 0; f < 6; ++f) {
    g.side_bc[f] = g.periodic[kAxisOf[f]] ? 0 : lv->side_bc[f];
    if (!g.periodic[kAxisOf[f]] && (g.side_bc[f] < 1 || g.side_bc[f] > 4))
      return set_err(ctx, FVGPU_ERR_ARG, "side_bc must be 1..4 on non-periodic sides");
  }
  cudaSetDevice(ctx->cfg.device);
  FV_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->drop_graphs();
  fv::reset_mixed(ctx->mixed);
  ctx->has_mesh = false;
  // pass 1: keys, 1:4 counts, record numbers
  DevBuf &d_level = ctx->lv_level, &d_ijk = ctx->lv_ijk, &d_keys = ctx->lv_keys, &d_off = ctx->lv_off,
         &d_tiles = ctx->lv_tiles, &d_scal = ctx->lv_scal;
  const int64_t ntiles = (n + 1023) / 1024;
  FV_CUDA(ctx, d_level.alloc(sizeof(int32_t) * size_t(n)));
  FV_CUDA(ctx, d_ijk.alloc(sizeof(int32_t) * 3 * size_t(n)));
  FV_CUDA(ctx, d_keys.alloc(sizeof(uint64_t) * size_t(n)));
  FV_CUDA(ctx, d_off.alloc(sizeof(int32_t) * size_t(n)));
  FV_CUDA(ctx, d_tiles.alloc(sizeof(int64_t) * size_t(ntiles)));
  FV_CUDA(ctx, d_scal.alloc(2 * sizeof(int64_t)));
  FV_CUDA(ctx, cudaMemcpy(d_level.p, lv->level, sizeof(int32_t) * size_t(n), cudaMemcpyHostToDevice));
  FV_CUDA(ctx, cudaMemcpy(d_ijk.p, lv->ijk, sizeof(int32_t) * 3 * size_t(n), cudaMemcpyHostToDevice));
  FV_CUDA(ctx, cudaMemset(d_scal.p, 0, 2 * sizeof(int64_t)));
  int64_t *d_nhang = d_scal.as<int64_t>();
  unsigned long long *d_ferr = reinterpret_cast<unsigned long long *>(d_scal.as<int64_t>() + 1);
  FV_CUDA(ctx, fv::flatten_count(g, n, d_level.as<int32_t>(), d_ijk.as<int32_t>(), d_keys.as<uint64_t>(),
                                 d_off.as<int32_t>(), d_tiles.as<int64_t>(), d_nhang, d_ferr, ctx->stream));
  int64_t hs[2] = {0, 0};
  FV_CUDA(ctx, cudaMemcpyAsync(hs, d_scal.p, sizeof hs, cudaMemcpyDeviceToHost, ctx->stream));
  FV_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  auto leaf_error = [&](uint64_t e) {
    const int code = int(e >> 40);
    const long long cell = (long long)(e & 0xffffffffffull);
    if (code == 1) return set_err(ctx, FVGPU_ERR_MESH, "leaf %lld: level or position out of range", cell);
    if (code == 2) return set_err(ctx, FVGPU_ERR_MESH, "leaves are not in Morton order (at %lld)", cell);
    return set_err(ctx, FVGPU_ERR_MESH, "leaf %lld: a face sees more than one level of refinement", cell);
  };
  if (hs[1]) return leaf_error(uint64_t(hs[1]));
  const int64_t nh = hs[0];
  if (nh > 6 * n) return set_err(ctx, FVGPU_ERR_MESH, "hanging-face count %lld out of range", (long long)nh);
  // pass 2: the tables, straight into the context's buffers
  for (DevBuf *b : {&ctx->nbr, &ctx->nbr_face}) FV_CUDA(ctx, b->alloc(sizeof(int32_t) * 6 * size_t(n)));
  for (DevBuf *b : {&ctx->area, &ctx->dcf, &ctx->dcc}) FV_CUDA(ctx, b->alloc(sizeof(double) * 6 * size_t(n)));
  FV_CUDA(ctx, ctx->vol.alloc(sizeof(double) * size_t(n)));
  FV_CUDA(ctx, ctx->level.alloc(sizeof(int32_t) * size_t(n)));
  FV_CUDA(ctx, ctx->hang_nbr.alloc(sizeof(int32_t) * 4 * size_t(nh)));
  FV_CUDA(ctx, ctx->hang_area.alloc(sizeof(double) * 4 * size_t(nh)));
  fv::DevTables t{ctx->nbr.as<int32_t>(), ctx->nbr_face.as<int32_t>(), ctx->hang_nbr.as<int32_t>(),
                  ctx->level.as<int32_t>(), ctx->area.as<double>(), ctx->dcf.as<double>(),
                  ctx->dcc.as<double>(), ctx->vol.as<double>(), ctx->hang_area.as<double>()};
  FV_CUDA(ctx, fv::flatten_tables(g, n, d_level.as<int32_t>(), d_ijk.as<int32_t>(), d_keys.as<uint64_t>(),
                                  d_off.as<int32_t>(), t, d_ferr, ctx->stream));
  FV_CUDA(ctx, cudaMemcpyAsync(hs, d_scal.p, sizeof hs, cudaMemcpyDeviceToHost, ctx->stream));
  FV_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (hs[1]) return leaf_error(uint64_t(hs[1]));
  // host copies for the signature, the boundary codes and the mixed path's brick detection
  const size_t un = static_cast<size_t>(n), unh = static_cast<size_t>(nh);
  const size_t n32 = 13 * un + 4 * unh, n64 = 19 * un + 4 * unh;  // int32: nbr, nbr_face, level, hang_nbr
  if (ctx->lv_h32.size() < n32) ctx->lv_h32.resize(n32);
  if (ctx->lv_h64.size() < n64) ctx->lv_h64.resize(n64);
  int32_t *h_nbr = ctx->lv_h32.data(), *h_nface = h_nbr + 6 * un, *h_level = h_nface + 6 * un,
          *h_hnbr = h_level + un;
  double *h_area = ctx->lv_h64.data(), *h_dcf = h_area + 6 * un, *h_dcc = h_dcf + 6 * un, *h_vol = h_dcc + 6 * un,
         *h_harea = h_vol + un;
  struct Down {
    void *dst;
    const DevBuf *src;
    size_t bytes;
  } downs[] = {{h_nbr, &ctx->nbr, 6 * un * 4},        {h_nface, &ctx->nbr_face, 6 * un * 4},
               {h_area, &ctx->area, 6 * un * 8},      {h_dcf, &ctx->dcf, 6 * un * 8},
               {h_dcc, &ctx->dcc, 6 * un * 8},        {h_vol, &ctx->vol, un * 8},
               {h_hnbr, &ctx->hang_nbr, 4 * unh * 4}, {h_harea, &ctx->hang_area, 4 * unh * 8},
               {h_level, &ctx->level, un * 4}};
  for (auto &d : downs)
    if (d.bytes) FV_CUDA(ctx, cudaMemcpy(d.dst, d.src->p, d.bytes, cudaMemcpyDeviceToHost));
  fvgpu_mesh_soa m{};
  m.ncells = n;
  m.nhang = nh;
  m.nbr = h_nbr;
  m.nbr_face = h_nface;
  m.area = h_area;
  m.dcf = h_dcf;
  m.dcc = h_dcc;
  m.vol = h_vol;
  m.hang_nbr = h_hnbr;
  m.hang_area = h_harea;
  m.frames = kBoxFrames.v;
  m.level = h_level;
  return finish_mesh(ctx, &m);
}

int fvgpu_upload_state(fvgpu_ctx *ctx, const double *U, int64_t ld) {
  int rc = ensure_state(ctx);
  if (rc) return rc;
  if (!U || ld < ctx->n) return set_err(ctx, FVGPU_ERR_ARG, "bad state pointer or leading dimension");
  cudaSetDevice(ctx->cfg.device);
  if (ld == ctx->n)  // dense: one linear copy
    FV_CUDA(ctx, cudaMemcpyAsync(ctx->S.p, U, sizeof(double) * ctx->neq * ctx->n, cudaMemcpyDefault,
                                 ctx->stream));
  else
    FV_CUDA(ctx, cudaMemcpy2DAsync(ctx->S.p, sizeof(double) * ctx->n, U, sizeof(double) * ld,
                                   sizeof(double) * ctx->n, ctx->neq, cudaMemcpyDefault, ctx->stream));
  ctx->lambda_valid = false;
  ctx->mixed.snf_valid = false;
  return FVGPU_OK;
}

int fvgpu_download_state(fvgpu_ctx *ctx, double *U, int64_t ld) {
  int rc = ensure_state(ctx);
  if (rc) return rc;
  if (!U || ld < ctx->n) return set_err(ctx, FVGPU_ERR_ARG, "bad state pointer or leading dimension");
  cudaSetDevice(ctx->cfg.device);
  if (ld == ctx->n)
    FV_CUDA(ctx, cudaMemcpyAsync(U, ctx->S.p, sizeof(double) * ctx->neq * ctx->n, cudaMemcpyDefault,
                                 ctx->stream));
  else
    FV_CUDA(ctx, cudaMemcpy2DAsync(U, sizeof(double) * ld, ctx->S.p, sizeof(double) * ctx->n,
                                   sizeof(double) * ctx->n, ctx->neq, cudaMemcpyDefault, ctx->stream));
  return sync_and_check(ctx);
}

int fvgpu_download(fvgpu_ctx *ctx, int field, double *out) {
  int rc = ensure_state(ctx);
  if (rc) return rc;
  if (!out) return set_err(ctx, FVGPU_ERR_ARG, "null output");
  cudaSetDevice(ctx->cfg.device);
  const DevBuf *b = nullptr;
  size_t bytes = 0;
  const int64_t n = ctx->n;
  switch (field) {
    case FVGPU_FIELD_S: b = &ctx->S; bytes = sizeof(double) * ctx->neq * n; break;
    case FVGPU_FIELD_SN: b = &ctx->SN; bytes = sizeof(double) * ctx->neq * n; break;
    case FVGPU_FIELD_RHS: b = &ctx->R; bytes = sizeof(double) * ctx->neq * n; break;
    case FVGPU_FIELD_SF:
      if (ctx->cfg.ischeme != 2) return set_err(ctx, FVGPU_ERR_STATE, "SF exists only for ischeme 2");
      b = &ctx->SF; bytes = sizeof(double) * 6 * ctx->neq * n; break;
    case FVGPU_FIELD_SG:
      bytes = sizeof(double) * (ctx->neq + 1) * 3 * n;
      if (ctx->SG.bytes < bytes) return set_err(ctx, FVGPU_ERR_STATE, "no gradients: call fvgpu_gradcalc first");
      b = &ctx->SG; break;
    default: return set_err(ctx, FVGPU_ERR_ARG, "unknown field %d", field);
  }
  FV_CUDA(ctx, cudaMemcpyAsync(out, b->p, bytes, cudaMemcpyDefault, ctx->stream));
  return sync_and_check(ctx);
}

int fvgpu_faceinterp(fvgpu_ctx *ctx) {
  int rc = ensure_state(ctx);
  if (rc) return rc;
  if (ctx->cfg.ischeme != 2) return set_err(ctx, FVGPU_ERR_STATE, "faceinterp needs ischeme 2");
  cudaSetDevice(ctx->cfg.device);
  return enqueue_faceinterp(ctx);
}

int fvgpu_gradcalc(fvgpu_ctx *ctx) {
  int rc = ensure_state(ctx);
  if (rc) return rc;
  cudaSetDevice(ctx->cfg.device);
  // inviscid runs allocate the gradients on first use (the host exports them,
  // loop.c:51)
  const size_t sg_bytes = sizeof(double) * size_t(ctx->neq + 1) * 3 * size_t(ctx->n);
  if (ctx->SG.bytes < sg_bytes) {
    FV_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    FV_CUDA(ctx, ctx->SG.alloc(sg_bytes));
    ctx->drop_graphs();  // graphs captured the old gradient buffer
  }
  return enqueue_gradcalc(ctx);
}

int fvgpu_rhs(fvgpu_ctx *ctx) {
  int rc = ensure_state(ctx);
  if (rc) return rc;
  cudaSetDevice(ctx->cfg.device);
  return enqueue_rhs(ctx, nullptr, 0);
}

int fvgpu_set_inner(fvgpu_ctx *ctx, const int32_t *inner) {
  int rc = ensure_state(ctx);
  if (rc) return rc;
  if (!inner) return set_err(ctx, FVGPU_ERR_ARG, "null inner flags");
  cudaSetDevice(ctx->cfg.device);
  FV_CUDA(ctx, ctx->inner.alloc(sizeof(int32_t) * ctx->n));
  FV_CUDA(ctx, cudaMemcpy(ctx->inner.p, inner, sizeof(int32_t) * ctx->n, cudaMemcpyHostToDevice));
  ctx->has_inner = true;
  return FVGPU_OK;
}

int fvgpu_rhs_nb(fvgpu_ctx *ctx, int inner_outer) {
  int rc = ensure_state(ctx);
  if (rc) return rc;
  if (!ctx->has_inner) return set_err(ctx, FVGPU_ERR_STATE, "fvgpu_set_inner not called");
  cudaSetDevice(ctx->cfg.device);
  return enqueue_rhs(ctx, ctx->inner.as<int32_t>(), inner_outer);
}

int fvgpu_rk(fvgpu_ctx *ctx, int irk, double dt) {
  int rc = ensure_state(ctx);
  if (rc) return rc;
  if (irk < 0 || irk > 4) return set_err(ctx, FVGPU_ERR_ARG, "irk must lie in 0..4");
  cudaSetDevice(ctx->cfg.device);
  k_set_double<<<1, 1, 0, ctx->stream>>>(ctx->d_dt(), dt);
  FV_LAUNCHED(ctx);
  fv::launch_rk_fp64(irk, ctx->ph, ctx->view(), ctx->S.as<double>(), ctx->SN.as<double>(), ctx->R.as<double>(),
                     ctx->d_dt(), nullptr, ctx->stream);
  FV_LAUNCHED(ctx);
  ctx->lambda_valid = false;
  ctx->mixed.snf_valid = false;
  return FVGPU_OK;
}

int fvgpu_compute_dt(fvgpu_ctx *ctx, double cfl, double *dt) {
  int rc = ensure_state(ctx);
  if (rc) return rc;
  if (!dt || !(cfl > 0.0)) return set_err(ctx, FVGPU_ERR_ARG, "need cfl > 0 and an output pointer");
  cudaSetDevice(ctx->cfg.device);
  FV_CUDA(ctx, cudaMemsetAsync(ctx->d_lambda_tmp(), 0, sizeof(double), ctx->stream));
  fv::launch_lambda_fp64(ctx->ph, ctx->view(), ctx->S.as<double>(), ctx->d_lambda_tmp(), ctx->stream);
  FV_LAUNCHED(ctx);
  FV_CUDA(ctx, cudaMemcpyAsync(&ctx->h_scal->lambda_tmp, ctx->d_lambda_tmp(), sizeof(double),
                               cudaMemcpyDeviceToHost, ctx->stream));
  rc = sync_and_check(ctx);
  if (rc) return rc;
  const double lam = ctx->h_scal->lambda_tmp;
  if (!(lam > 0.0) || !std::isfinite(lam)) return set_err(ctx, FVGPU_ERR_NONFINITE, "spectral radius %g", lam);
  *dt = cfl / lam;
  return FVGPU_OK;
}

int fvgpu_step(fvgpu_ctx *ctx, int scheme, double dt, double cfl, int nsteps) {
  int rc = ensure_state(ctx);
  if (rc) return rc;
  if (scheme < FVGPU_SCHEME_EULER || scheme > FVGPU_SCHEME_SSPRK3 || nsteps < 0)
    return set_err(ctx, FVGPU_ERR_ARG, "bad scheme or step count");
  const bool cfl_mode = !(dt > 0.0);
  if (cfl_mode && !(cfl > 0.0)) return set_err(ctx, FVGPU_ERR_ARG, "dt <= 0 needs cfl > 0");
  cudaSetDevice(ctx->cfg.device);
  if (nsteps == 0) return FVGPU_OK;
  if (cfl_mode) {
    rc = ensure_lambda(ctx);  // mixed: also refreshes the FP32 copy
    if (rc) return rc;
  }
  rc = ensure_mixed_f32(ctx);
  if (rc) return rc;
  if (cfl_mode) {
    k_set_double<<<1, 1, 0, ctx->stream>>>(&ctx->d_scal()->cfl, cfl);
  } else {
    k_set_double<<<1, 1, 0, ctx->stream>>>(ctx->d_dt(), dt);
  }
  FV_LAUNCHED(ctx);
  for (int s = 0; s < nsteps; ++s) {
  const GraphKey key{scheme, cfl_mode ? 1 : 0, ctx->cfg.precision, ctx->S.p};
  auto it = ctx->graphs.find(key);
  if (it == ctx->graphs.end()) {
    cudaGraph_t g = nullptr;
    int before = 0;
    for (int k = 0; k < FVGPU_NKINDS; ++k) before += ctx->marks.counts[k];
    FV_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    rc = enqueue_step(ctx, scheme, cfl_mode);
    int after = 0;
    for (int k = 0; k < FVGPU_NKINDS; ++k) after += ctx->marks.counts[k];
    ctx->graph_launches[key] = after - before;
    cudaError_t ce = cudaStreamEndCapture(ctx->stream, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (ce != cudaSuccess) return set_err(ctx, FVGPU_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
    cudaGraphExec_t ge = nullptr;
    ce = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return set_err(ctx, FVGPU_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ce));
    it = ctx->graphs.emplace(key, ge).first;
  }
  FV_CUDA(ctx, cudaGraphLaunch(it->second, ctx->stream));
  after_step(ctx);
  }
  if (!cfl_mode) ctx->lambda_valid = false;
  return FVGPU_OK;
}

int fvgpu_profile_step(fvgpu_ctx *ctx, int scheme, double dt, double cfl, int nsteps, double *ms,
                       int *launches) {
  int rc = ensure_state(ctx);
  if (rc) return rc;
  if (!ms || !launches || nsteps <= 0) return set_err(ctx, FVGPU_ERR_ARG, "need outputs and nsteps > 0");
  if (scheme < FVGPU_SCHEME_EULER || scheme > FVGPU_SCHEME_SSPRK3) return set_err(ctx, FVGPU_ERR_ARG, "bad scheme");
  const bool cfl_mode = !(dt > 0.0);
  if (cfl_mode && !(cfl > 0.0)) return set_err(ctx, FVGPU_ERR_ARG, "dt <= 0 needs cfl > 0");
  cudaSetDevice(ctx->cfg.device);
  if (cfl_mode) {
    rc = ensure_lambda(ctx);  // mixed: also refreshes the FP32 copy
    if (rc) return rc;
  }
  rc = ensure_mixed_f32(ctx);
  if (rc) return rc;
  if (cfl_mode) {
    k_set_double<<<1, 1, 0, ctx->stream>>>(&ctx->d_scal()->cfl, cfl);
  } else {
    k_set_double<<<1, 1, 0, ctx->stream>>>(ctx->d_dt(), dt);
  }
  FV_LAUNCHED(ctx);
  const int cap = 64 * nsteps + 2;
  std::vector<cudaEvent_t> ev(size_t(cap), nullptr);
  std::vector<int> kinds(size_t(cap), -1);
  for (auto &e : ev) FV_CUDA(ctx, cudaEventCreate(&e));
  fv::LaunchMarks &mk = ctx->marks;
  mk.active = true;
  mk.stream = ctx->stream;
  mk.events = ev.data();
  mk.kinds = kinds.data();
  mk.capacity = cap - 1;
  mk.used = 0;
  for (int s = 0; s < nsteps && rc == 0; ++s) {
    rc = enqueue_step(ctx, scheme, cfl_mode);
    if (!rc) after_step(ctx);
  }
  const int used = mk.used;
  cudaEventRecord(ev[size_t(used)], ctx->stream);
  mk.active = false;
  mk.events = nullptr;
  mk.kinds = nullptr;
  if (!rc) rc = sync_and_check(ctx);
  for (int k = 0; k < FVGPU_NKINDS; ++k) {
    ms[k] = 0.0;
    launches[k] = 0;
  }
  if (!rc) {
    for (int i = 0; i < used; ++i) {
      float t = 0.f;
      cudaEventElapsedTime(&t, ev[size_t(i)], ev[size_t(i) + 1]);
      ms[kinds[size_t(i)]] += double(t);
      launches[kinds[size_t(i)]] += 1;
    }
  }
  for (auto &e : ev) cudaEventDestroy(e);
  if (!cfl_mode) ctx->lambda_valid = false;
  return rc;
}

int fvgpu_get_stream(fvgpu_ctx *ctx, void **stream) {
  if (!ctx || !stream) return FVGPU_ERR_ARG;
  *stream = (void *)ctx->stream;
  return FVGPU_OK;
}

int fvgpu_conservation(fvgpu_ctx *ctx, double *sums) {
  int rc = ensure_state(ctx);
  if (rc) return rc;
  if (!sums) return set_err(ctx, FVGPU_ERR_ARG, "null output");
  cudaSetDevice(ctx->cfg.device);
  double *part = ctx->partial.as<double>();
  k_cons_partial<<<kConsBlocks, kConsThreads, 0, ctx->stream>>>(ctx->neq, ctx->n, ctx->S.as<double>(),
                                                                ctx->vol.as<double>(), part);
  FV_LAUNCHED(ctx);
  double *d_sums = part + kConsBlocks * (fv::kNeqMax + 1);  // 8 spare slots after the block rows
  k_cons_final<<<1, kConsThreads, 0, ctx->stream>>>(ctx->neq, part, d_sums);
  FV_LAUNCHED(ctx);
  FV_CUDA(ctx, cudaMemcpyAsync(sums, d_sums, sizeof(double) * (ctx->neq + 1), cudaMemcpyDeviceToHost,
                               ctx->stream));
  return sync_and_check(ctx);
}

// ---- restart files ---------------------------------------------------------------------

namespace {
struct CkHeader {
  char magic[8];
  uint32_t version, neq;
  int64_t ncells;
  uint64_t mesh_sig;
  double time;
  int64_t step;
};
static_assert(sizeof(CkHeader) == 48, "restart header layout");
}  // namespace

int fvgpu_checkpoint_write(const char *path, const double *U, int neq, int64_t ncells, uint64_t mesh_sig,
                           double time, int64_t step) {
  if (!path || !U || neq <= 0 || ncells <= 0) return FVGPU_ERR_ARG;
  CkHeader h{};
  memcpy(h.magic, "FVGPUCK1", 8);
  h.version = 1;
  h.neq = uint32_t(neq);
  h.ncells = ncells;
  h.mesh_sig = mesh_sig;
  h.time = time;
  h.step = step;
  const size_t bytes = sizeof(double) * size_t(neq) * size_t(ncells);
  const uint64_t sum = fnv1a(fnv1a(kFnvSeed, &h, sizeof h), U, bytes);
  FILE *f = fopen(path, "wb");
  if (!f) return FVGPU_ERR_ARG;
  const bool ok = fwrite(&h, sizeof h, 1, f) == 1 && fwrite(U, 1, bytes, f) == bytes && fwrite(&sum, 8, 1, f) == 1;
  return (fclose(f) == 0 && ok) ? FVGPU_OK : FVGPU_ERR_ARG;
}

int fvgpu_checkpoint_read(const char *path, double *U, int neq, int64_t ncells, uint64_t mesh_sig, double *time,
                          int64_t *step) {
  if (!path || !U || neq <= 0 || ncells <= 0) return FVGPU_ERR_ARG;
  FILE *f = fopen(path, "rb");
  if (!f) return FVGPU_ERR_ARG;
  CkHeader h{};
  const size_t bytes = sizeof(double) * size_t(neq) * size_t(ncells);
  uint64_t sum = 0;
  int rc = FVGPU_OK;
  if (fread(&h, sizeof h, 1, f) != 1 || memcmp(h.magic, "FVGPUCK1", 8) != 0 || h.version != 1)
    rc = FVGPU_ERR_STATE;
  else if (h.neq != uint32_t(neq) || h.ncells != ncells || h.mesh_sig != mesh_sig)
    rc = FVGPU_ERR_STATE;
  else if (fread(U, 1, bytes, f) != bytes || fread(&sum, 8, 1, f) != 1)
    rc = FVGPU_ERR_STATE;
  else if (fgetc(f) != EOF || sum != fnv1a(fnv1a(kFnvSeed, &h, sizeof h), U, bytes))
    rc = FVGPU_ERR_STATE;
  fclose(f);
  if (rc == FVGPU_OK) {
    if (time) *time = h.time;
    if (step) *step = h.step;
  }
  return rc;
}

// FNV-1a over the resident tables, in the order and over the bytes the
// upload received them (counts, neighbour codes and faces, areas, volumes,
// 1:4 records, levels); formed once per mesh, on first use, from device copies.
static int ensure_mesh_sig(fvgpu_ctx *ctx) {
  if (ctx->mesh_sig_valid) return FVGPU_OK;
  const int64_t n = ctx->n, nh = ctx->nhang;
  cudaSetDevice(ctx->cfg.device);
  FV_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  uint64_t h = kFnvSeed;
  h = fnv1a(h, &n, sizeof(int64_t));
  h = fnv1a(h, &nh, sizeof(int64_t));
  std::vector<unsigned char> buf;
  auto add = [&](const DevBuf &b, size_t bytes) -> cudaError_t {
    buf.resize(bytes);
    const cudaError_t e = cudaMemcpy(buf.data(), b.p, bytes, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) h = fnv1a(h, buf.data(), bytes);
    return e;
  };
  FV_CUDA(ctx, add(ctx->nbr, sizeof(int32_t) * 6 * size_t(n)));
  FV_CUDA(ctx, add(ctx->nbr_face, sizeof(int32_t) * 6 * size_t(n)));
  FV_CUDA(ctx, add(ctx->area, sizeof(double) * 6 * size_t(n)));
  FV_CUDA(ctx, add(ctx->vol, sizeof(double) * size_t(n)));
  if (nh > 0) {
    FV_CUDA(ctx, add(ctx->hang_nbr, sizeof(int32_t) * 4 * size_t(nh)));
    FV_CUDA(ctx, add(ctx->hang_area, sizeof(double) * 4 * size_t(nh)));
  }
  if (ctx->mesh_has_level) FV_CUDA(ctx, add(ctx->level, sizeof(int32_t) * size_t(n)));
  ctx->mesh_sig = h;
  ctx->mesh_sig_valid = true;
  return FVGPU_OK;
}

int fvgpu_mesh_signature(fvgpu_ctx *ctx, uint64_t *sig) {
  int rc = ensure_state(ctx);
  if (rc) return rc;
  if (!sig) return set_err(ctx, FVGPU_ERR_ARG, "null output");
  if ((rc = ensure_mesh_sig(ctx))) return rc;
  *sig = ctx->mesh_sig;
  return FVGPU_OK;
}

int fvgpu_checkpoint_save(fvgpu_ctx *ctx, const char *path, double time, int64_t step) {
  int rc = ensure_state(ctx);
  if (rc) return rc;
  std::vector<double> U(size_t(ctx->neq) * size_t(ctx->n));
  rc = fvgpu_download_state(ctx, U.data(), ctx->n);
  if (rc) return rc;
  if ((rc = ensure_mesh_sig(ctx))) return rc;
  rc = fvgpu_checkpoint_write(path, U.data(), ctx->neq, ctx->n, ctx->mesh_sig, time, step);
  return rc ? set_err(ctx, rc, "cannot write restart file %s", path ? path : "(null)") : FVGPU_OK;
}

int fvgpu_checkpoint_load(fvgpu_ctx *ctx, const char *path, double *time, int64_t *step) {
  int rc = ensure_state(ctx);
  if (rc) return rc;
  if ((rc = ensure_mesh_sig(ctx))) return rc;
  std::vector<double> U(size_t(ctx->neq) * size_t(ctx->n));
  rc = fvgpu_checkpoint_read(path, U.data(), ctx->neq, ctx->n, ctx->mesh_sig, time, step);
  if (rc) return set_err(ctx, rc, "restart file %s does not match this mesh or is damaged", path ? path : "(null)");
  rc = fvgpu_upload_state(ctx, U.data(), ctx->n);
  if (rc) return rc;
  return sync_and_check(ctx);
}

int fvgpu_criterion(fvgpu_ctx *ctx, int kind, double threshold, int32_t level_hi, int32_t *split) {
  int rc = ensure_state(ctx);
  if (rc) return rc;
  if (!split || kind < FVGPU_CRIT_GRAD_RHO || kind > FVGPU_CRIT_GRAD_RHO_H)
    return set_err(ctx, FVGPU_ERR_ARG, "bad criterion or output");
  const size_t sg_bytes = sizeof(double) * size_t(ctx->neq + 1) * 3 * size_t(ctx->n);
  if (kind != FVGPU_CRIT_RHO_BELOW && ctx->SG.bytes < sg_bytes)
    return set_err(ctx, FVGPU_ERR_STATE, "no gradients: call fvgpu_gradcalc first");
  cudaSetDevice(ctx->cfg.device);
  DevBuf flags;
  FV_CUDA(ctx, flags.alloc(sizeof(int32_t) * size_t(ctx->n)));
  const unsigned blocks = unsigned(std::min<int64_t>((ctx->n + 255) / 256, 4096));
  k_criterion<<<blocks, 256, 0, ctx->stream>>>(kind, threshold, level_hi, ctx->n, ctx->S.as<double>(),
                                               ctx->SG.as<double>(), ctx->vol.as<double>(), flags.as<int32_t>());
  FV_LAUNCHED(ctx);
  FV_CUDA(ctx, cudaMemcpyAsync(split, flags.p, sizeof(int32_t) * size_t(ctx->n), cudaMemcpyDeviceToHost,
                               ctx->stream));
  return sync_and_check(ctx);
}

int fvgpu_halo_set(fvgpu_ctx *ctx, const int32_t *send_cells, int64_t nsend, const int32_t *recv_cells,
                   int64_t nrecv) {
  int rc = ensure_state(ctx);
  if (rc) return rc;
  if (nsend < 0 || nrecv < 0 || (nsend > 0 && !send_cells) || (nrecv > 0 && !recv_cells))
    return set_err(ctx, FVGPU_ERR_ARG, "bad halo lists");
  std::vector<uint8_t> seen(size_t(ctx->n), 0);
  for (int64_t i = 0; i < nsend; ++i)
    if (send_cells[i] < 0 || send_cells[i] >= ctx->n) return set_err(ctx, FVGPU_ERR_ARG, "send cell %lld out of range", (long long)i);
  for (int64_t i = 0; i < nrecv; ++i) {
    const int32_t c = recv_cells[i];
    if (c < 0 || c >= ctx->n) return set_err(ctx, FVGPU_ERR_ARG, "recv cell %lld out of range", (long long)i);
    if (seen[size_t(c)]) return set_err(ctx, FVGPU_ERR_ARG, "recv cell %d listed twice", c);
    seen[size_t(c)] = 1;
  }
  cudaSetDevice(ctx->cfg.device);
  FV_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  FV_CUDA(ctx, ctx->halo_send.alloc(sizeof(int32_t) * size_t(nsend)));
  FV_CUDA(ctx, ctx->halo_recv.alloc(sizeof(int32_t) * size_t(nrecv)));
  if (nsend) FV_CUDA(ctx, cudaMemcpy(ctx->halo_send.p, send_cells, sizeof(int32_t) * size_t(nsend), cudaMemcpyHostToDevice));
  if (nrecv) FV_CUDA(ctx, cudaMemcpy(ctx->halo_recv.p, recv_cells, sizeof(int32_t) * size_t(nrecv), cudaMemcpyHostToDevice));
  ctx->nsend = nsend;
  ctx->nrecv = nrecv;
  return FVGPU_OK;
}

int fvgpu_halo_pack(fvgpu_ctx *ctx, double *send_buf) {
  int rc = ensure_state(ctx);
  if (rc) return rc;
  if (ctx->nsend == 0) return FVGPU_OK;
  if (!send_buf) return set_err(ctx, FVGPU_ERR_ARG, "null send buffer");
  cudaSetDevice(ctx->cfg.device);
  const unsigned blocks = unsigned(std::min<int64_t>((ctx->nsend + 255) / 256, 1024));
  k_halo_gather<<<blocks, 256, 0, ctx->stream>>>(ctx->neq, ctx->n, ctx->S.as<double>(), ctx->halo_send.as<int32_t>(),
                                                 ctx->nsend, send_buf);
  FV_LAUNCHED(ctx);
  return FVGPU_OK;
}

int fvgpu_halo_unpack(fvgpu_ctx *ctx, const double *recv_buf) {
  int rc = ensure_state(ctx);
  if (rc) return rc;
  if (ctx->nrecv == 0) return FVGPU_OK;
  if (!recv_buf) return set_err(ctx, FVGPU_ERR_ARG, "null receive buffer");
  cudaSetDevice(ctx->cfg.device);
  const unsigned blocks = unsigned(std::min<int64_t>((ctx->nrecv + 255) / 256, 1024));
  k_halo_scatter<<<blocks, 256, 0, ctx->stream>>>(ctx->neq, ctx->n, ctx->S.as<double>(), ctx->halo_recv.as<int32_t>(),
                                                  ctx->nrecv, recv_buf);
  FV_LAUNCHED(ctx);
  ctx->lambda_valid = false;
  ctx->mixed.snf_valid = false;
  return FVGPU_OK;
}

int fvgpu_residual_vjp(fvgpu_ctx *ctx, const double *w, double *dJdU, int64_t ld) {
  int rc = ensure_state(ctx);
  if (rc) return rc;
  if (!w || !dJdU || ld < ctx->n) return set_err(ctx, FVGPU_ERR_ARG, "bad array pointer or leading dimension");
  cudaSetDevice(ctx->cfg.device);
  rc = ensure_adjoint(ctx);
  if (rc) return rc;
  const size_t row = sizeof(double) * size_t(ctx->n);
  FV_CUDA(ctx, cudaMemcpy2DAsync(ctx->adjW.p, row, w, sizeof(double) * ld, row, ctx->neq, cudaMemcpyDefault,
                                 ctx->stream));
  rc = enqueue_vjp(ctx, ctx->S.as<double>(), ctx->adjW.as<double>(), ctx->adjG.as<double>());
  if (rc) return rc;
  FV_CUDA(ctx, cudaMemcpy2DAsync(dJdU, sizeof(double) * ld, ctx->adjG.p, row, row, ctx->neq,
                                 cudaMemcpyDefault, ctx->stream));
  return sync_and_check(ctx);
}

int fvgpu_residual_vjp_device(fvgpu_ctx *ctx, const double *w, double *dJdU) {
  int rc = ensure_state(ctx);
  if (rc) return rc;
  if (!w || !dJdU) return set_err(ctx, FVGPU_ERR_ARG, "null array");
  cudaSetDevice(ctx->cfg.device);
  rc = ensure_adjoint(ctx);
  if (rc) return rc;
  return enqueue_vjp(ctx, ctx->S.as<double>(), w, dJdU);
}

int fvgpu_adjoint_steps(fvgpu_ctx *ctx, int scheme, double dt, int nsteps, const double *gN, double *g0,
                        int64_t ld) {
  int rc = ensure_state(ctx);
  if (rc) return rc;
  if (scheme < FVGPU_SCHEME_EULER || scheme > FVGPU_SCHEME_SSPRK3 || nsteps < 0 || !(dt > 0.0) ||
      !std::isfinite(dt))
    return set_err(ctx, FVGPU_ERR_ARG, "need a scheme, nsteps >= 0 and a finite dt > 0");
  if (!gN || !g0 || ld < ctx->n) return set_err(ctx, FVGPU_ERR_ARG, "bad array pointer or leading dimension");
  cudaSetDevice(ctx->cfg.device);
  rc = ensure_adjoint(ctx);
  if (rc) return rc;
  const size_t row = sizeof(double) * size_t(ctx->n);
  const size_t cell = row * size_t(ctx->neq);
  if (ctx->adj_ck_steps < nsteps) {
    FV_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    FV_CUDA(ctx, ctx->adjCK.alloc(cell * size_t(nsteps)));
    ctx->adj_ck_steps = nsteps;
  }
  k_set_double<<<1, 1, 0, ctx->stream>>>(ctx->d_dt(), dt);
  FV_LAUNCHED(ctx);
  // forward sweep: checkpoint, then the step itself (the FP64 sequence fvgpu_step runs)
  char *ck = static_cast<char *>(ctx->adjCK.p);
  for (int k = 0; k < nsteps; ++k) {
    FV_CUDA(ctx, cudaMemcpyAsync(ck + cell * size_t(k), ctx->S.p, cell, cudaMemcpyDeviceToDevice, ctx->stream));
    rc = enqueue_step_fp64(ctx, scheme, false);
    if (rc) return rc;
  }
  ctx->mixed.snf_valid = false;
  ctx->lambda_valid = false;
  // reverse sweep
  FV_CUDA(ctx, cudaMemcpy2DAsync(ctx->adjG.p, row, gN, sizeof(double) * ld, row, ctx->neq, cudaMemcpyDefault,
                                 ctx->stream));
  for (int k = nsteps - 1; k >= 0; --k) {
    rc = enqueue_step_adjoint(ctx, scheme, reinterpret_cast<const double *>(ck + cell * size_t(k)));
    if (rc) return rc;
  }
  FV_CUDA(ctx, cudaMemcpy2DAsync(g0, sizeof(double) * ld, ctx->adjG.p, row, row, ctx->neq, cudaMemcpyDefault,
                                 ctx->stream));
  return sync_and_check(ctx);
}

int fvgpu_profile_adjoint(fvgpu_ctx *ctx, int reps, double *ms_residual, double *ms_vjp) {
  int rc = ensure_state(ctx);
  if (rc) return rc;
  if (reps <= 0 || !ms_residual || !ms_vjp) return set_err(ctx, FVGPU_ERR_ARG, "need reps > 0 and outputs");
  cudaSetDevice(ctx->cfg.device);
  rc = ensure_adjoint(ctx);
  if (rc) return rc;
  const size_t cell = sizeof(double) * size_t(ctx->neq) * size_t(ctx->n);
  // residual weights: the state itself (any dense field exercises every path)
  FV_CUDA(ctx, cudaMemcpyAsync(ctx->adjW.p, ctx->S.p, cell, cudaMemcpyDeviceToDevice, ctx->stream));
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  for (auto &e : ev) FV_CUDA(ctx, cudaEventCreate(&e));
  for (int pass = 0; pass < 2 && rc == 0; ++pass) {
    const int n = pass == 0 ? 1 : reps;
    if (pass == 1) cudaEventRecord(ev[0], ctx->stream);
    for (int i = 0; i < n && rc == 0; ++i) {
      if (ctx->cfg.ischeme == 2) rc = enqueue_faceinterp(ctx);
      if (!rc && ctx->cfg.ns == 1) rc = enqueue_gradcalc(ctx);
      if (!rc) rc = enqueue_rhs(ctx, nullptr, 0);
    }
    if (pass == 1) cudaEventRecord(ev[1], ctx->stream);
    for (int i = 0; i < n && rc == 0; ++i)
      rc = enqueue_vjp(ctx, ctx->S.as<double>(), ctx->adjW.as<double>(), ctx->adjG.as<double>());
    if (pass == 1) cudaEventRecord(ev[2], ctx->stream);
  }
  if (!rc) rc = sync_and_check(ctx);
  if (!rc) {
    float t0 = 0.f, t1 = 0.f;
    cudaEventElapsedTime(&t0, ev[0], ev[1]);
    cudaEventElapsedTime(&t1, ev[1], ev[2]);
    *ms_residual = double(t0) / reps;
    *ms_vjp = double(t1) / reps;
  }
  for (auto &e : ev) cudaEventDestroy(e);
  return rc;
}

int fvgpu_synchronize(fvgpu_ctx *ctx) {
  if (!ctx) return FVGPU_ERR_ARG;
  cudaSetDevice(ctx->cfg.device);
  return sync_and_check(ctx);
}

int fvgpu_last_error(fvgpu_ctx *ctx, int *code, int64_t *cell, char *msg, int msglen) {
  const std::string &m = ctx ? ctx->last_msg : g_create_error;
  if (code) *code = ctx ? ctx->last_code : 0;
  if (cell) *cell = ctx ? ctx->last_cell : -1;
  if (msg && msglen > 0) {
    strncpy(msg, m.c_str(), size_t(msglen) - 1);
    msg[msglen - 1] = 0;
  }
  return FVGPU_OK;
}

}  // extern "C"
