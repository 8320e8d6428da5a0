/*
 * fvgpu.h -- C ABI of libfvgpu: the residual evaluation and Runge-Kutta stage
 * update of the octree finite-volume solver FV_140823, on one GB300 (sm_103a).
 *
 * The reference path is, per RK stage (the stage sequence of the missing
 * driver advancetimeexplicit, loop.c:48):
 *     faceinterp(run)                 faceinterp.c:21-61   (MUSCL, ischeme 2)
 *     gradcalc(run)                   gradcalc.c:9-47      (viscous, ns 1)
 *     RHS(run) / RHS_nb(run, inner)   RHS.c:3-13, RHS_nb.c:3-15
 *        -> residual_faces_AMR        residual_faces_AMR.c:10-202
 *     RK(irk, run)                    RK.c:3-56
 * all of them `void` functions over the host leaf list `run->topo->locl`.
 * Here the host flattens its leaves once per adaptation (fvgpu_mesh_soa),
 * uploads them with fvgpu_upload_mesh, and the state stays resident in HBM;
 * each reference call has a counterpart below that works on the resident
 * state.  Reference semantics kept exactly: operation order per cell and
 * face (the FP64 path is bit-identical to the reference up to its use of
 * libm pow(x, 2.0), for which the correctly rounded x*x is used), the stage
 * formulas of RK.c, boundary codes of bc.c, EOS models 1-3.
 *
 * Conventions
 *   - every call returns FVGPU_OK (0) or a negative FVGPU_ERR_* code; the
 *     reference instead printf()s and calls exit(0) (residual_faces_AMR.c:
 *     186-194, hllc_euler.c:52-55, compute_wave_speeds.c:84-87);
 *   - kernels never trap: a non-finite residual or a failed EOS sets a device
 *     error word (first cell + code), which the next synchronising call turns
 *     into FVGPU_ERR_NONFINITE / FVGPU_ERR_EOS; fvgpu_last_error() reports it;
 *   - host buffers are caller-owned; device buffers belong to the context;
 *   - state arrays are structure-of-arrays, U[v * ld + c] for variable v of
 *     cell c (ld >= ncells);
 *   - one context per host thread; each context owns one CUDA stream.  On
 *     an AMR mesh a mixed-precision stage forks part of its work to a second
 *     internal stream and joins it back before the stage ends, so every call
 *     is still ordered on (and capturable from) the context's stream.
 */
#ifndef FVGPU_H
#define FVGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FVGPU_OK 0
#define FVGPU_ERR_ARG (-1)          /* invalid argument */
#define FVGPU_ERR_CUDA (-2)         /* CUDA runtime error (message in fvgpu_last_error) */
#define FVGPU_ERR_NOMEM (-3)        /* device allocation failed */
#define FVGPU_ERR_STATE (-4)        /* call order (e.g. no mesh uploaded) */
#define FVGPU_ERR_NONFINITE (-5)    /* a residual / state became NaN or Inf */
#define FVGPU_ERR_EOS (-6)          /* mixture EOS has no real pressure root */
#define FVGPU_ERR_UNSUPPORTED (-7)  /* configuration the library does not implement */
#define FVGPU_ERR_MESH (-8)         /* mesh tables failed validation at upload */
#define FVGPU_ERR_NODEVICE (-9)     /* no CUDA device */
#define FVGPU_ERR_TIMEOUT (-10)     /* a bounded device wait gave up */

/* arithmetic of the residual */
#define FVGPU_FP64 0   /* everything in FP64, reference operation order */
#define FVGPU_MIXED 1  /* reconstruction, EOS, gradients and fluxes (HLLC and
                          viscous) in FP32; residual accumulation, RK update,
                          sums, dt and the mixture-EOS pressure in FP64 */

/* fvgpu_config.flags */
#define FVGPU_FLAG_NO_BRICKS 1  /* mixed path: run every cell through the general
                                   (table-driven) kernel instead of the brick
                                   kernel; results are bit-identical */

/* RK schemes = stage lists of RK(irk) (RK.c:16-47) */
#define FVGPU_SCHEME_EULER 1   /* RK(0), RK(1) */
#define FVGPU_SCHEME_SSPRK2 2  /* RK(0), RK(1), RK(4) */
#define FVGPU_SCHEME_SSPRK3 3  /* RK(0), RK(1), RK(2), RK(3) */

/* what fvgpu_download() copies */
#define FVGPU_FIELD_S 0    /* state S            [neq][ncells] */
#define FVGPU_FIELD_SN 1   /* step-start state SN [neq][ncells] */
#define FVGPU_FIELD_RHS 2  /* residual RHS       [neq][ncells] */
#define FVGPU_FIELD_SF 3   /* MUSCL face values SF [6][neq][ncells] */
#define FVGPU_FIELD_SG 4   /* gradients SG       [neq+1][3][ncells] */

/* Neighbour code per (face, cell), as in the mesh builder (fvmesh.h):
 * >= 0 neighbour cell; -1-bc for a boundary face (bc 1..4, bc.c:19-49);
 * <= FVGPU_HANG0: 1:4 hanging face, record FVGPU_HANG0 - code. */
#define FVGPU_HANG0 (-16)

/* Solver constants read by the residual path (CON / PAR, strdata.h:199-358;
 * positional .ct input, inputset.c:39-110). */
typedef struct fvgpu_config {
  int model;       /* 1 ideal/stiffened gas, 2 barotropic liquid, 3 two-phase mixture */
  int ns;          /* 1 = viscous (Navier-Stokes) fluxes */
  int ischeme;     /* 1 first order, 2 MUSCL / minmod */
  int iprimtv;     /* must be 0: MUSCL on the conservative variables
                      (reconctruct_V3.c, iprimtv == 0); the primitive-variable
                      branch is not provided */
  int eos;         /* 1 = viscous work term in the energy flux (flux_viscous.c:227) */
  int precision;   /* FVGPU_FP64 or FVGPU_MIXED */
  int device;      /* CUDA device ordinal */
  int flags;       /* FVGPU_FLAG_* */
  double gamma;    /* PAR.matergama[0] */
  double pinf;     /* PAR.materpinf[0] */
  double visc;     /* PAR.matervisc[0] */
  double ymin;     /* CON.ymin (mass-fraction clip of facercnstr.c:43-44) */
  double inflow[8];/* conservative ghost state of bc code 1 (bc_inlet.c) */
  double reserved[4];
} fvgpu_config;

/* Flattened mesh, structure of arrays ([face][cell] = f * ncells + c). */
typedef struct fvgpu_mesh_soa {
  int64_t ncells;
  int64_t nhang;
  const int32_t *nbr;       /* [6][ncells] neighbour code */
  const int32_t *nbr_face;  /* [6][ncells] neighbour's face index (neigfc), -1 at boundaries */
  const double *area;       /* [6][ncells] Area[f][0] of single-neighbour / boundary faces */
  const double *dcf;        /* [6][ncells] distance.c dist_cf of face f */
  const double *dcc;        /* [6][ncells] distance.c dist_cc of face f */
  const double *vol;        /* [ncells] */
  const int32_t *hang_nbr;  /* [nhang][4] fine neighbours of a 1:4 face, sub-face order */
  const double *hang_area;  /* [nhang][4] Area[f][0..3] of a 1:4 face */
  const double *frames;     /* [6][9] face frame per face index: n, t1, t2 */
  const int32_t *level;     /* [ncells] octree level (used by the mixed path) */
} fvgpu_mesh_soa;

typedef struct fvgpu_ctx fvgpu_ctx;

/* ---- lifetime --------------------------------------------------------- */
int fvgpu_create(const fvgpu_config *cfg, fvgpu_ctx **out);
int fvgpu_destroy(fvgpu_ctx *ctx);
/* Switch FP64 <-> mixed arithmetic; keeps mesh and state. */
int fvgpu_set_precision(fvgpu_ctx *ctx, int precision);

/* ---- data in / out ---------------------------------------------------- */
/* Validates and uploads the tables (once per adaptation); resets the state. */
int fvgpu_upload_mesh(fvgpu_ctx *ctx, const fvgpu_mesh_soa *mesh);
/* Device-side flattening: builds the tables of fvgpu_upload_mesh on the GPU
 * from the leaf list of an axis-aligned box -- the level and the integer
 * position (i, j, k at that level) of every leaf, leaves 2:1 balanced and in
 * Morton order -- with the host builder's arithmetic (fvmesh_flatten of
 * fvmesh.h), so the tables are the same bit for bit.  The host keeps its
 * octree and uploads 16 bytes per leaf after an adaptation instead of
 * flattening on the CPU.  No reference counterpart (the reference walks its
 * leaf list in every call).  FVGPU_ERR_MESH for unsorted, out-of-range or
 * unbalanced leaves. */
typedef struct fvgpu_leaves {
  int64_t ncells;
  const int32_t *level;  /* [ncells] */
  const int32_t *ijk;    /* [3][ncells] */
  double lo[3], len[3];  /* the box */
  int periodic[3];       /* per axis */
  int side_bc[6];        /* boundary code per face side (ignored on periodic axes) */
} fvgpu_leaves;
int fvgpu_upload_leaves(fvgpu_ctx *ctx, const fvgpu_leaves *leaves);
/* S <- U ([neq][ld]); LEAF.S of every leaf (strdata.h:80).  U may be host
 * or device memory (the copy direction follows from unified addressing); the
 * copy is queued on the context's stream. */
int fvgpu_upload_state(fvgpu_ctx *ctx, const double *U, int64_t ld);
int fvgpu_download_state(fvgpu_ctx *ctx, double *U, int64_t ld);
/* Copy a device field (FVGPU_FIELD_*) to host or device memory (densely
 * packed). */
int fvgpu_download(fvgpu_ctx *ctx, int field, double *out);

/* ---- the reference's calls -------------------------------------------- */
/* faceinterp(run), faceinterp.c:21-61: SF from S. */
int fvgpu_faceinterp(fvgpu_ctx *ctx);
/* gradcalc(run), gradcalc.c:9-47: SG from S (for ns == 0 the gradient
 * array is allocated on the first call, as the host exports gradients). */
int fvgpu_gradcalc(fvgpu_ctx *ctx);
/* RHS(run), RHS.c:3-13: RHS from S, SF, SG (as the reference, faceinterp /
 * gradcalc must have been called first when ischeme == 2 / ns == 1). */
int fvgpu_rhs(fvgpu_ctx *ctx);
/* RHS_nb(run, inner_outer), RHS_nb.c:3-15: RHS of the cells whose inner flag
 * equals inner_outer (flags from fvgpu_set_inner; inner_el.c:3-30). */
int fvgpu_set_inner(fvgpu_ctx *ctx, const int32_t *inner);
int fvgpu_rhs_nb(fvgpu_ctx *ctx, int inner_outer);
/* RK(irk, run), RK.c:3-56, with CON.dt = dt. */
int fvgpu_rk(fvgpu_ctx *ctx, int irk, double dt);

/* ---- fused time stepping ---------------------------------------------- */
/* nsteps full RK steps (scheme FVGPU_SCHEME_*).  dt > 0: fixed step (the
 * reference's CON.dt).  dt <= 0: each step uses the CFL step
 *     dt = cfl / max_c (sum_faces A (|u.n| + c)) / (2 V)
 * reduced on the device from the step-start state.  Each step is one CUDA
 * graph launch. */
int fvgpu_step(fvgpu_ctx *ctx, int scheme, double dt, double cfl, int nsteps);
/* dt = cfl / lambda_max of the current state (no state change). */
int fvgpu_compute_dt(fvgpu_ctx *ctx, double cfl, double *dt);
/* sums[v] = sum_c S[v][c] * V[c] (v < neq), sums[neq] = sum_c V[c]
 * (conservationcalc.c:19-34), FP64, fixed reduction order. */
int fvgpu_conservation(fvgpu_ctx *ctx, double *sums);

/* Conservation sums for callers that cannot allocate device memory (no
 * counterpart in the reference).  Some host codes reserve all their device
 * memory up front and allow no allocation inside the time loop, or run under
 * a device-memory cap that is already fully committed; they cannot give
 * fvgpu_conservation the context-owned scratch it allocates.  This variant
 * takes DEVICE pointers the caller owns -- S [neq][ncells], vol [ncells] and
 * sums [neq+1] -- and keeps its scratch in a fixed 48 KiB device array of the
 * library (every GPU that loads the library holds it until exit).  Limits:
 * 1 <= neq <= 5, 1 <= ncells < 2^31, else FVGPU_ERR_ARG.  It allocates
 * nothing.  The first call on a device, and the first after that device's
 * context was destroyed and created again (cudaDeviceReset), looks up the
 * array's device address: make it before any stream capture on that device.
 * All calls share the
 * array: calls that overlap on the GPU race, so order them.  Work is queued on
 * `stream` (a cudaStream_t, NULL = default stream); sums are ready when that
 * stream reaches this point. */
int fvgpu_conservation_noalloc(const double *S, const double *vol, int64_t ncells, int neq, double *sums,
                               void *stream);

/* ---- restart and adaptation helpers ------------------------------------ */
/* Bit-exact binary restart of the state.  The reference writes its restart
 * as "%15.10e" text (restart_save.c:41, restart_load.c), which drops about
 * five significant digits; this file holds the FP64 state as stored: header
 * {magic "FVGPUCK1", version 1, neq, ncells, mesh signature (FNV-1a of the
 * uploaded neighbour, level, area and volume tables), time, step}, the state
 * [neq][ncells] as little-endian doubles, then an FNV-1a checksum of the
 * payload.  fvgpu_checkpoint_load rejects a file whose checksum, size or mesh
 * signature does not match the context (FVGPU_ERR_STATE). */
int fvgpu_checkpoint_save(fvgpu_ctx *ctx, const char *path, double time, int64_t step);
int fvgpu_checkpoint_load(fvgpu_ctx *ctx, const char *path, double *time, int64_t *step);
/* The same format on host arrays, without a context (tools, tests). */
int fvgpu_checkpoint_write(const char *path, const double *U, int neq, int64_t ncells, uint64_t mesh_sig,
                           double time, int64_t step);
int fvgpu_checkpoint_read(const char *path, double *U, int neq, int64_t ncells, uint64_t mesh_sig, double *time,
                          int64_t *step);
/* Mesh signature of the context's uploaded tables. */
int fvgpu_mesh_signature(fvgpu_ctx *ctx, uint64_t *sig);

/* Refinement flags from the current state (criterionsplt.c:24-86): split[c]
 * = level_hi where the criterion holds, else 1 (the reference's default).
 *   FVGPU_CRIT_GRAD_RHO   |grad rho| > threshold (i_case 204; the gradients
 *                         of the last fvgpu_gradcalc, row 0 of SG)
 *   FVGPU_CRIT_RHO_BELOW  rho < threshold (i_case 2500)
 *   FVGPU_CRIT_GRAD_RHO_H |grad rho| * h > threshold, h = V^(1/3) (the
 *                         cell-size-scaled form used to build AMR cases)
 * split: host array [ncells]. */
#define FVGPU_CRIT_GRAD_RHO 0
#define FVGPU_CRIT_RHO_BELOW 1
#define FVGPU_CRIT_GRAD_RHO_H 2
int fvgpu_criterion(fvgpu_ctx *ctx, int kind, double threshold, int32_t level_hi, int32_t *split);

/* ---- halo exchange (domain decomposition) ------------------------------- */
/* The reference exchanges the state of interface cells between MPI ranks
 * once per stage (communicate_S, communicate1.c:44-229).  Here a rank's mesh
 * holds its own cells plus a 2-deep ghost layer (fv_140823_gb300/halo.py
 * builds both and the lists below); before each stage the owner packs the
 * cells other ranks hold as ghosts, the caller moves the buffers (NCCL,
 * MPI, or a copy between contexts on one GPU) and the receiver unpacks them
 * into its ghost cells.  Index lists are host arrays of local cell indices,
 * copied at the call; recv_cells must be distinct.  Buffers are DEVICE arrays
 * [neq][count] the caller owns; pack and unpack are queued on the context's
 * stream (fvgpu_get_stream).  FP64 state only. */
int fvgpu_halo_set(fvgpu_ctx *ctx, const int32_t *send_cells, int64_t nsend, const int32_t *recv_cells,
                   int64_t nrecv);
int fvgpu_halo_pack(fvgpu_ctx *ctx, double *send_buf);
int fvgpu_halo_unpack(fvgpu_ctx *ctx, const double *recv_buf);

/* ---- adjoint ----------------------------------------------------------- */
/* No reference counterpart: the reference has no derivative code.  These
 * entry points give the transpose of the FP64 residual and step maps
 * (residual_faces_AMR.c with hllc_euler.c, faceinterp.c / reconctruct_V3.c,
 * RK.c), computed by hand-written reverse kernels: deterministic (gathers in a
 * fixed order, no atomics).  Scope: model 1, inviscid or viscous (the
 * reverse of flux_viscous and of the Green-Gauss gradients it reads, turb =
 * 0), first order or MUSCL, boundary codes other than the walls 3 and 4;
 * other configurations return FVGPU_ERR_UNSUPPORTED.  Derivatives are those of the branch the forward
 * takes at the given state (minmod, wave-speed and HLLC-region choices); at a
 * branch switch they are one-sided.  In a context on the FP32-mixed path
 * (FVGPU_MIXED) the reverse passes run in FP32: face values, flux, limiter
 * and EOS reversed in FP32 with FP32 intermediate sums, linearised at the
 * FP64 state (the multi-step adjoint recomputes its stage states with FP64
 * steps); weights, the viscous gradients and the result stay FP64. */

/* dJdU = (dR/dU)^T w for the residual R(U) of the current state; w and dJdU
 * arrays [neq][ld] in host or device memory.  The context's SF field then
 * holds the face values of the current state. */
int fvgpu_residual_vjp(fvgpu_ctx *ctx, const double *w, double *dJdU, int64_t ld);

/* The same on device arrays [neq][ncells] the caller owns, queued on the
 * context's stream (fvgpu_get_stream) with no host copy or synchronisation. */
int fvgpu_residual_vjp_device(fvgpu_ctx *ctx, const double *w, double *dJdU);

/* Multi-step adjoint with one checkpoint per RK step.  From the current
 * state S_0 it runs nsteps FP64 steps of `scheme` at the fixed time step dt
 * (dt is a constant of the map, not a function of the state), keeping every
 * step-start state on the device (nsteps * neq * ncells doubles, grown on
 * demand and kept for reuse), then sweeps back: each step's stage states are
 * recomputed from its checkpoint and the stages are reversed.  On return the
 * current state is S_N, exactly as fvgpu_step(ctx, scheme, dt, 0, nsteps)
 * leaves it, and g0 = (dS_N/dS_0)^T gN.  gN and g0 are arrays [neq][ld] in
 * host or device memory; they may be the same array. */
int fvgpu_adjoint_steps(fvgpu_ctx *ctx, int scheme, double dt, int nsteps, const double *gN, double *g0,
                        int64_t ld);

/* Device time of the residual and of its adjoint on the current state: reps
 * eager launches of each (FP64 face values + residual, then face values +
 * the three reverse passes), timed with CUDA events on the context's stream
 * after one untimed round; mean milliseconds per evaluation. */
int fvgpu_profile_adjoint(fvgpu_ctx *ctx, int reps, double *ms_residual, double *ms_vjp);

/* ---- diagnostics -------------------------------------------------------- */
/* Measurement utility, not part of the solver path (no reference
 * counterpart): the FP64 arithmetic rate of the device in G operations/s,
 * from separate adds and multiplies in registers on every SM, as the FP64
 * path issues them.  bench.py divides the FP64 residual's counted operations
 * by it for that kernel's roofline fraction. */
int fvgpu_measure_fp64(int device, double *gops);

/* Kernel kinds reported by fvgpu_profile_step. */
#define FVGPU_KIND_FACEINTERP 0  /* faceinterp.c */
#define FVGPU_KIND_GRADCALC 1    /* gradcalc.c */
#define FVGPU_KIND_RESIDUAL 2    /* residual_faces_AMR.c (+ fused RK stage) */
#define FVGPU_KIND_RK 3          /* RK.c */
#define FVGPU_KIND_DT 4          /* CFL spectral radius / time step */
#define FVGPU_KIND_MIXED_STAGE 5 /* mixed path: fused reconstruction + flux + RK stage */
#define FVGPU_KIND_MIXED_AUX 6   /* mixed path: auxiliary kernels */
#define FVGPU_KIND_ADJOINT 7     /* residual adjoint (reverse passes) */
#define FVGPU_NKINDS 8
/* Run nsteps steps eagerly (no graph) with a CUDA event recorded on the
 * context's stream before every kernel and after the last; ms[k] receives the
 * summed device time of kind k and launches[k] its launch count (arrays of
 * FVGPU_NKINDS).  Same arguments and results as fvgpu_step. */
int fvgpu_profile_step(fvgpu_ctx *ctx, int scheme, double dt, double cfl, int nsteps, double *ms,
                       int *launches);
/* The CUDA stream (cudaStream_t) all of the context's work is queued on. */
int fvgpu_get_stream(fvgpu_ctx *ctx, void **stream);
/* Error of the last failing call: code, offending cell (-1 if none) and text. */
int fvgpu_last_error(fvgpu_ctx *ctx, int *code, int64_t *cell, char *msg, int msglen);
/* Number of conserved variables of the configured model (5 or 4). */
int fvgpu_neq(const fvgpu_ctx *ctx);
/* Block until all work queued on the context's stream has finished. */
int fvgpu_synchronize(fvgpu_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif
