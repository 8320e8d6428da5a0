/*
 * fvshim.c -- link-time drop-in of libfvgpu for the FV_140823 host program
 * (interface and sync points in include/fvshim.h).
 *
 * Built with the host's own include path (strdata.h and the MPI / METIS /
 * PETSc headers it includes) and linked into the host executable instead of
 * RHS.o, RHS_nb.o, RK.o, faceinterp.o and gradcalc.o.
 *
 * Flattening follows the fvgpu_mesh_soa contract of include/fvgpu.h from the
 * fields the reference's residual reads (residual_faces_AMR.c:29-130):
 *   cl->fc[f].bc != 0           boundary face, code -1 - bc
 *   lfc_neigs[f] == 1           single neighbour neigtr[f][0], its face neigfc[f]
 *   lfc_neigs[f] == 4           1:4 face, fine neighbours neigtr[f][0..3]
 *   cl->Area[f][s], cl->Vol     areas and volume
 *   cl->nx..nzt2[f]             face frames (one table for the whole mesh)
 *   distance(run, crnt, f, ..)  MUSCL distances, the host's own distance.c
 * Neighbours are identified by their LEAF (periodic or proxy branches share
 * the real leaf's storage, forestconn.c:36-57).
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "strdata.h"

#include "fvgpu.h"
#include "fvshim.h"

typedef struct {
  const void *key;
  int64_t idx;
} slot_t;

static struct {
  fvgpu_ctx *ctx;
  RUN *run;
  int64_t n, nhang;
  BRANCH **leaf;
  slot_t *map;
  size_t mapcap;
  /* flattened tables (host copies kept for re-use of their buffers) */
  int32_t *nbr, *nbr_face, *hang_nbr, *level, *inner;
  double *area, *dcf, *dcc, *vol, *hang_area, *U;
  double frames[54];
  int scheme, precision;
  int need_mesh, need_state, has_inner;
  int has_grad; /* the device holds gradients of the current leaves */
  long uploads, syncs;
  void (*handler)(int, const char *);
} G = {.scheme = 0, .precision = FVGPU_FP64, .need_mesh = 1, .need_state = 1};

/* ---- errors ----------------------------------------------------------------- */

static void fail(int code, const char *what) {
  char msg[600];
  char lib[512] = {0};
  int c = 0;
  int64_t cell = -1;
  fvgpu_last_error(G.ctx, &c, &cell, lib, (int)sizeof lib);
  snprintf(msg, sizeof msg, "fvshim: %s failed (%d): %s", what, code, lib);
  if (G.handler) {
    G.handler(code, msg);
    return;
  }
  printf("%s\n", msg);
  exit(0); /* the reference's reaction to a failed residual */
}

#define CHECK(call, what)     \
  do {                        \
    int rc_ = (call);         \
    if (rc_ != FVGPU_OK) {    \
      fail(rc_, what);        \
      return;                 \
    }                         \
  } while (0)

/* ---- LEAF -> index map --------------------------------------------------------- */

static size_t hash_ptr(const void *p) {
  uint64_t x = (uint64_t)(uintptr_t)p;
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  return (size_t)x;
}

static void *grow(void *p, size_t bytes) {
  void *q = realloc(p, bytes ? bytes : 16);
  if (!q) {
    printf("fvshim: out of host memory\n");
    exit(0);
  }
  return q;
}

static void map_reset(int64_t n) {
  size_t cap = 16;
  while (cap < (size_t)(2 * n + 1)) cap <<= 1;
  if (cap != G.mapcap) {
    G.map = grow(G.map, cap * sizeof(slot_t));  /* exits with a message when out of memory */
    G.mapcap = cap;
  }
  for (size_t i = 0; i < cap; ++i) G.map[i].key = NULL;
}

static void map_put(const void *key, int64_t idx) {
  size_t i = hash_ptr(key) & (G.mapcap - 1);
  while (G.map[i].key != NULL && G.map[i].key != key) i = (i + 1) & (G.mapcap - 1);
  G.map[i].key = key;
  G.map[i].idx = idx;
}

static int64_t map_get(const void *key) {
  size_t i = hash_ptr(key) & (G.mapcap - 1);
  while (G.map[i].key != NULL) {
    if (G.map[i].key == key) return G.map[i].idx;
    i = (i + 1) & (G.mapcap - 1);
  }
  return -1;
}

/* ---- flattening ---------------------------------------------------------------- */


/* Builds the tables from run->topo->locl; returns 0 or a message. */
static const char *flatten(RUN *run) {
  int64_t n = 0, nh = 0;
  for (BRANCH *b = run->topo->locl; b != NULL; b = b->lnxt) {
    ++n;
    if (b->nlfc != 6) return "only hexahedral leaves (6 faces) are supported";
    for (int f = 0; f < 6; ++f)
      if (b->cl->fc[f].bc == 0 && b->lfc_neigs[f] != 1) {
        if (b->lfc_neigs[f] != 4) return "a face with neither 1 nor 4 neighbours";
        ++nh;
      }
  }
  if (n == 0) return "empty leaf list";
  G.n = n;
  G.nhang = nh;
  G.leaf = grow(G.leaf, (size_t)n * sizeof(BRANCH *));
  G.nbr = grow(G.nbr, (size_t)(6 * n) * sizeof(int32_t));
  G.nbr_face = grow(G.nbr_face, (size_t)(6 * n) * sizeof(int32_t));
  G.area = grow(G.area, (size_t)(6 * n) * sizeof(double));
  G.dcf = grow(G.dcf, (size_t)(6 * n) * sizeof(double));
  G.dcc = grow(G.dcc, (size_t)(6 * n) * sizeof(double));
  G.vol = grow(G.vol, (size_t)n * sizeof(double));
  G.level = grow(G.level, (size_t)n * sizeof(int32_t));
  G.hang_nbr = grow(G.hang_nbr, (size_t)(4 * nh) * sizeof(int32_t));
  G.hang_area = grow(G.hang_area, (size_t)(4 * nh) * sizeof(double));
  map_reset(n);
  int64_t c = 0;
  for (BRANCH *b = run->topo->locl; b != NULL; b = b->lnxt, ++c) {
    G.leaf[c] = b;
    map_put(b->el, c);
  }
  /* one face-frame table: the first leaf's, every leaf must agree */
  const CELL *c0 = G.leaf[0]->cl;
  for (int f = 0; f < 6; ++f) {
    double *fr = G.frames + 9 * f;
    fr[0] = c0->nx[f];
    fr[1] = c0->ny[f];
    fr[2] = c0->nz[f];
    fr[3] = c0->nxt1[f];
    fr[4] = c0->nyt1[f];
    fr[5] = c0->nzt1[f];
    fr[6] = c0->nxt2[f];
    fr[7] = c0->nyt2[f];
    fr[8] = c0->nzt2[f];
  }
  int64_t r = 0;
  for (c = 0; c < n; ++c) {
    BRANCH *b = G.leaf[c];
    CELL *cl = b->cl;
    G.level[c] = b->level;
    G.vol[c] = cl->Vol;
    for (int f = 0; f < 6; ++f) {
      const double *fr = G.frames + 9 * f;
      if (cl->nx[f] != fr[0] || cl->ny[f] != fr[1] || cl->nz[f] != fr[2] || cl->nxt1[f] != fr[3] ||
          cl->nyt1[f] != fr[4] || cl->nzt1[f] != fr[5] || cl->nxt2[f] != fr[6] || cl->nyt2[f] != fr[7] ||
          cl->nzt2[f] != fr[8])
        return "leaves with different face frames";
      const int64_t i = (int64_t)f * n + c;
      double cf = 0.0, cc = 0.0;
      distance(run, b, f, &cf, &cc);
      G.dcf[i] = cf;
      G.dcc[i] = cc;
      if (cl->fc[f].bc != 0) {
        G.nbr[i] = -1 - cl->fc[f].bc;
        G.nbr_face[i] = -1;
        G.area[i] = cl->Area[f][0];
      } else if (b->lfc_neigs[f] == 1) {
        const int64_t k = map_get(b->neigtr[f][0]->el);
        if (k < 0) return "a neighbour outside the leaf list";
        G.nbr[i] = (int32_t)k;
        G.nbr_face[i] = b->neigfc[f];
        G.area[i] = cl->Area[f][0];
      } else {
        G.nbr[i] = (int32_t)(FVGPU_HANG0 - r);
        G.nbr_face[i] = b->neigfc[f];
        G.area[i] = 0.0;
        for (int s = 0; s < 4; ++s) {
          const int64_t k = map_get(b->neigtr[f][s]->el);
          if (k < 0) return "a fine neighbour outside the leaf list";
          G.hang_nbr[4 * r + s] = (int32_t)k;
          G.hang_area[4 * r + s] = cl->Area[f][s];
        }
        ++r;
      }
    }
  }
  return NULL;
}

/* ---- context ------------------------------------------------------------------- */

static void make_config(RUN *run, fvgpu_config *cfg) {
  memset(cfg, 0, sizeof *cfg);
  const CON *con = run->con;
  cfg->model = con->model;
  cfg->ns = con->ns;
  cfg->ischeme = con->ischeme;
  cfg->iprimtv = con->iprimtv;
  cfg->eos = con->eos;
  cfg->precision = G.precision;
  cfg->device = 0;
  cfg->gamma = run->par->matergama[0];
  cfg->pinf = run->par->materpinf[0];
  cfg->visc = run->par->matervisc[0];
  cfg->ymin = con->ymin;
  /* inflow ghost state: the host's own bc_inlet (bc_inlet.c, by i_case) */
  for (int64_t c = 0; c < G.n; ++c) {
    BRANCH *b = G.leaf[c];
    for (int f = 0; f < 6; ++f)
      if (b->cl->fc[f].bc == 1) {
        bc_inlet(b, f, run);
        for (int v = 0; v < con->neq && v < 8; ++v) cfg->inflow[v] = run->sol1->vec[v];
        return;
      }
  }
}

static void gather_state(RUN *run) {
  const int neq = run->con->neq;
  G.U = grow(G.U, (size_t)(neq * G.n) * sizeof(double));
  for (int64_t c = 0; c < G.n; ++c)
    for (int v = 0; v < neq; ++v) G.U[(int64_t)v * G.n + c] = G.leaf[c]->el->S[v];
}

static void ensure(RUN *run) {
  if (G.run != run) {
    fvshim_release();
    G.run = run;
  }
  if (G.need_mesh) {
    const char *why = flatten(run);
    if (why) {
      printf("fvshim: cannot flatten the leaf list: %s\n", why);
      if (G.handler) {
        G.handler(FVGPU_ERR_MESH, why);
        return;
      }
      exit(0);
    }
    if (!G.ctx) {
      fvgpu_config cfg;
      make_config(run, &cfg);
      CHECK(fvgpu_create(&cfg, &G.ctx), "fvgpu_create");
    }
    fvgpu_mesh_soa m;
    memset(&m, 0, sizeof m);
    m.ncells = G.n;
    m.nhang = G.nhang;
    m.nbr = G.nbr;
    m.nbr_face = G.nbr_face;
    m.area = G.area;
    m.dcf = G.dcf;
    m.dcc = G.dcc;
    m.vol = G.vol;
    m.hang_nbr = G.hang_nbr;
    m.hang_area = G.hang_area;
    m.frames = G.frames;
    m.level = G.level;
    CHECK(fvgpu_upload_mesh(G.ctx, &m), "fvgpu_upload_mesh");
    G.uploads++;
    G.need_mesh = 0;
    G.need_state = 1;
    G.has_inner = 0;
    G.has_grad = 0;
  }
  if (G.need_state) {
    gather_state(run);
    CHECK(fvgpu_upload_state(G.ctx, G.U, G.n), "fvgpu_upload_state");
    G.need_state = 0;
  }
}

/* ---- the reference's symbols ------------------------------------------------------ */

void faceinterp(struct RUN *run) {
  ensure(run);
  CHECK(fvgpu_faceinterp(G.ctx), "faceinterp");
}

void gradcalc(struct RUN *run) {
  ensure(run);
  CHECK(fvgpu_gradcalc(G.ctx), "gradcalc");
  G.has_grad = 1;
  /* the host calls gradcalc itself before exporting fields (loop.c:51) */
  fvshim_sync_host(run, FVSHIM_S | FVSHIM_SG);
}

void RHS(struct RUN *run) {
  ensure(run);
  CHECK(fvgpu_rhs(G.ctx), "RHS");
}

void RHS_nb(struct RUN *run, int inner_outer) {
  ensure(run);
  if (!G.has_inner) {
    G.inner = grow(G.inner, (size_t)G.n * sizeof(int32_t));
    for (int64_t c = 0; c < G.n; ++c) G.inner[c] = G.leaf[c]->el->inner;
    CHECK(fvgpu_set_inner(G.ctx, G.inner), "fvgpu_set_inner");
    G.has_inner = 1;
  }
  CHECK(fvgpu_rhs_nb(G.ctx, inner_outer), "RHS_nb");
}

void RK(int irk, RUN *run) {
  ensure(run);
  CHECK(fvgpu_rk(G.ctx, irk, run->con->dt), "RK");
}

/* One time step of con->dt (loop.c:48); the loop itself advances con->time
 * and con->istep (Init_clocks.c:70-71). */
void advancetimeexplicit(struct RUN *run) {
  const CON *con = run->con;
  /* loop.c runs meshadaptation right before this call on adaptation steps */
  if (con->adapth != 0 && con->adapthstep > 0 && con->istep % con->adapthstep == 0 && G.uploads > 0)
    fvshim_invalidate(run);
  ensure(run);
  const int scheme = G.scheme ? G.scheme : (con->method == 1 || con->method == 2 ? con->method : FVGPU_SCHEME_SSPRK3);
  CHECK(fvgpu_step(G.ctx, scheme, con->dt, 0.0, 1), "advancetimeexplicit");
  if (con->ns == 1) G.has_grad = 1;
  const int next = con->istep + 1;
  const int restart = con->ststep > 0 && next % con->ststep == 0;
  const int adapt = con->adapth != 0 && con->adapthstep > 0 && next % con->adapthstep == 0;
  if (restart || adapt) fvshim_sync_host(run, FVSHIM_S);
}

void advancetimeexplicit_nb(struct RUN *run) { advancetimeexplicit(run); }

/* ---- shim controls ---------------------------------------------------------------- */

void fvshim_sync_host(struct RUN *run, int fields) {
  if (!G.ctx || G.run != run || G.need_mesh) return; /* the leaves are authoritative */
  const int neq = run->con->neq;
  const int64_t n = G.n;
  static const struct {
    int bit, field, rows;
  } kinds[] = {{FVSHIM_S, FVGPU_FIELD_S, 1}, {FVSHIM_SN, FVGPU_FIELD_SN, 1}, {FVSHIM_RHS, FVGPU_FIELD_RHS, 1},
               {FVSHIM_SF, FVGPU_FIELD_SF, 6}, {FVSHIM_SG, FVGPU_FIELD_SG, 3}};
  for (size_t k = 0; k < sizeof kinds / sizeof kinds[0]; ++k) {
    if (!(fields & kinds[k].bit)) continue;
    if (kinds[k].bit == FVSHIM_SF && run->con->ischeme != 2) continue;
    if (kinds[k].bit == FVSHIM_SG && !G.has_grad) continue; /* nothing computed them yet */
    const int64_t per = kinds[k].bit == FVSHIM_SF ? 6 * neq : (kinds[k].bit == FVSHIM_SG ? 3 * (neq + 1) : neq);
    G.U = grow(G.U, (size_t)(per * n) * sizeof(double));
    CHECK(fvgpu_download(G.ctx, kinds[k].field, G.U), "fvgpu_download");
    for (int64_t c = 0; c < n; ++c) {
      LEAF *el = G.leaf[c]->el;
      switch (kinds[k].bit) {
        case FVSHIM_S:
          for (int v = 0; v < neq; ++v) el->S[v] = G.U[(int64_t)v * n + c];
          break;
        case FVSHIM_SN:
          for (int v = 0; v < neq; ++v) el->SN[v] = G.U[(int64_t)v * n + c];
          break;
        case FVSHIM_RHS:
          for (int v = 0; v < neq; ++v) el->RHS[v] = G.U[(int64_t)v * n + c];
          break;
        case FVSHIM_SF:
          for (int f = 0; f < 6; ++f)
            for (int v = 0; v < neq; ++v) el->SF[f][v] = G.U[((int64_t)f * neq + v) * n + c];
          break;
        default:
          for (int v = 0; v <= neq; ++v)
            for (int d = 0; d < 3; ++d) el->SG[v][d] = G.U[((int64_t)v * 3 + d) * n + c];
          break;
      }
    }
  }
  G.syncs++;
}

void fvshim_invalidate(struct RUN *run) {
  (void)run;
  G.need_mesh = 1;
  G.need_state = 1;
}

void fvshim_set_scheme(int scheme) { G.scheme = scheme; }

void fvshim_set_precision(int precision) {
  G.precision = precision;
  if (G.ctx && fvgpu_set_precision(G.ctx, precision) != FVGPU_OK) fail(FVGPU_ERR_UNSUPPORTED, "set_precision");
}

void fvshim_set_error_handler(void (*handler)(int code, const char *msg)) { G.handler = handler; }

void fvshim_release(void) {
  if (G.ctx) fvgpu_destroy(G.ctx);
  G.ctx = NULL;
  G.run = NULL;
  G.need_mesh = 1;
  G.need_state = 1;
  G.has_inner = 0;
}

void fvshim_counters(long *uploads, long *syncs) {
  if (uploads) *uploads = G.uploads;
  if (syncs) *syncs = G.syncs;
}
