/*
 * ref_harness.c -- runs the reference's own residual / RK code on a mesh
 * given as flattened tables.  TEST INFRASTRUCTURE ONLY: it is linked with the
 * reference's hot-path sources, compiled unchanged (oracle/build.py), into
 * oracle/_ref/libfvref.so, and is loaded only by tests/ and by the fixture
 * generator under tests/golden/.
 *
 * The reference cannot run as shipped (its time-step driver
 * advancetimeexplicit, loop.c:48, is missing, and so are brchconn,
 * cellallocation, bc_reflective and bc_wall).  This harness supplies:
 *   - a serial MPI_Wtime / MPI_Allreduce / MPI_Barrier, and MPI_Send /
 *     MPI_Recv that a single process never reaches;
 *   - bc_reflective / bc_wall as no-ops (the reference declares them,
 *     bc.c:38,42, but defines neither);
 *   - the BRANCH / CELL / LEAF objects the residual walks, built directly from
 *     the tables (bypassing brchconn / cellallocation): leaf list
 *     `run->topo->locl`, `neigtr/lfc_neigs/neigfc/nsfc`, parent branches for
 *     distance.c, a level-0 `glob` branch for boundary faces, and periodic
 *     image branches that share the real leaf's state but carry translated
 *     node coordinates (the reference has no periodic boundary; this mirrors
 *     its proxy "keen" branches, forestconn.c:36-57);
 *   - the stage sequence of the missing driver: RK(0), then per stage
 *     faceinterp (MUSCL) -> gradcalc (viscous) -> RHS -> RK(k);
 *   - the forest the Tecplot writer walks (refh_export).
 * Leaf storage (LEAF.S, SN, RHS, SF, SG) is allocated by the reference's own
 * memallocation.c / leafallocation.c, scratch by createutility.c.
 * Node coordinates use the mesh builder's rule x = lo + I * (len / 2^level).
 */
#include "strdata.h"

#include <stdint.h>
#include <time.h>

/* ---- serial MPI stand-ins --------------------------------------------- */
double MPI_Wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype dt, MPI_Op op, MPI_Comm c) {
  size_t w = dt == MPI_DOUBLE ? sizeof(double) : (dt == MPI_LONG ? sizeof(long) : sizeof(int));
  (void)op;
  (void)c;
  memmove(r, s, (size_t)n * w);
  return 0;
}
int MPI_Barrier(MPI_Comm c) {
  (void)c;
  return 0;
}
/* Point-to-point calls: a single process has no peer.  The writer and the
 * halo exchange only reach them when run->con->size > 1. */
int MPI_Send(const void *b, int n, MPI_Datatype dt, int dest, int tag, MPI_Comm c) {
  (void)b, (void)n, (void)dt, (void)dest, (void)tag, (void)c;
  fprintf(stderr, "ref_harness: MPI_Send in a serial run\n");
  return 1;
}
int MPI_Recv(void *b, int n, MPI_Datatype dt, int src, int tag, MPI_Comm c, MPI_Status *st) {
  (void)b, (void)n, (void)dt, (void)src, (void)tag, (void)c, (void)st;
  fprintf(stderr, "ref_harness: MPI_Recv in a serial run\n");
  return 1;
}

/* ---- reference symbols that are declared but never defined -------------- */
void bc_reflective(struct BRANCH *crnt, int f, RUN *run) {
  (void)crnt;
  (void)f;
  (void)run;
}
void bc_wall(struct BRANCH *crnt, int f, struct RUN *run) {
  (void)crnt;
  (void)f;
  (void)run;
}

/* ---- harness ------------------------------------------------------------- */
typedef struct refh_config {
  int model, ns, ischeme, iprimtv, neq, eos, i_case, pad;
  double gamma, pinf, visc, ymin, dt;
} refh_config;

typedef struct refh {
  RUN *run;
  int64_t n;
  BRANCH **cells;
  BRANCH *glob;
  BRANCH **extra; /* parents and images, kept for teardown */
  int64_t nextra, capextra;
  double lo[3], len[3];
  int periodic[3];
  int32_t *ijk; /* [3][n] leaf positions, for the export's forest */
} refh;

static const int kAxis[6] = {1, 0, 1, 0, 2, 2};
static const int kSign[6] = {-1, +1, +1, -1, -1, +1};

static double coordv(const refh *h, int level, int a, int64_t I) {
  return h->lo[a] + (double)I * ldexp(h->len[a], -level);
}

static CELL *make_cell_nodes(const refh *h, int level, const int64_t p[3]) {
  CELL *cl = calloc(1, sizeof(CELL));
  cl->nd = calloc(8, sizeof(ND));
  for (int n = 0; n < 8; ++n) {
    cl->nd[n].num = n;
    cl->nd[n].x = coordv(h, level, 0, p[0] + (n & 1));
    cl->nd[n].y = coordv(h, level, 1, p[1] + ((n >> 1) & 1));
    cl->nd[n].z = coordv(h, level, 2, p[2] + ((n >> 2) & 1));
  }
  return cl;
}

static void keep(refh *h, BRANCH *b) {
  if (h->nextra == h->capextra) {
    h->capextra = h->capextra ? 2 * h->capextra : 1024;
    h->extra = realloc(h->extra, (size_t)h->capextra * sizeof(BRANCH *));
  }
  h->extra[h->nextra++] = b;
}

static int64_t fdiv2(int64_t a) { return a >= 0 ? a / 2 : -((-a + 1) / 2); }

/* Parent branch: distance.c only reads its node coordinates and node count
 * (distance.c:163-171, 182-190). */
static BRANCH *make_parent(refh *h, int level, const int64_t p[3]) {
  BRANCH *b = calloc(1, sizeof(BRANCH));
  int64_t q[3] = {fdiv2(p[0]), fdiv2(p[1]), fdiv2(p[2])};
  b->level = level - 1;
  b->nlnd = 8;
  b->nlfc = 6;
  b->cl = make_cell_nodes(h, level - 1, q);
  keep(h, b);
  return b;
}

/* Periodic image of a real branch at the unwrapped position p: same leaf
 * (state), translated nodes and parent. */
static BRANCH *make_image(refh *h, BRANCH *real, const int64_t p[3]) {
  BRANCH *b = calloc(1, sizeof(BRANCH));
  *b = *real;
  b->cl = make_cell_nodes(h, real->level, p);
  b->prnt = make_parent(h, real->level, p);
  keep(h, b);
  return b;
}

/* Branch to use for neighbour `idx` when the unwrapped position at its level
 * is `up`: the real branch, or an image if the link wraps around. */
static BRANCH *neighbour_branch(refh *h, int64_t idx, const int32_t *ijk, const int64_t up[3]) {
  BRANCH *real = h->cells[idx];
  int64_t n = h->n;
  if (ijk[idx] == up[0] && ijk[n + idx] == up[1] && ijk[2 * n + idx] == up[2]) return real;
  return make_image(h, real, up);
}

refh *refh_create(const refh_config *cfg, int64_t n, const int32_t *level, const int32_t *ijk,
                  const int32_t *nbr, const int32_t *nbr_face, const double *area,
                  const double *vol, const double *centroid, const int32_t *hang_nbr,
                  const double *hang_area, const double *frames, const double lo[3],
                  const double len[3], const int periodic[3]) {
  refh *h = calloc(1, sizeof(refh));
  for (int a = 0; a < 3; ++a) {
    h->lo[a] = lo[a];
    h->len[a] = len[a];
    h->periodic[a] = periodic[a];
  }
  h->n = n;
  h->ijk = malloc((size_t)(3 * (n > 0 ? n : 1)) * sizeof(int32_t));
  memcpy(h->ijk, ijk, (size_t)(3 * n) * sizeof(int32_t));
  RUN *run = calloc(1, sizeof(RUN));
  h->run = run;
  run->con = calloc(1, sizeof(CON));
  run->par = calloc(1, sizeof(PAR));
  run->sol = calloc(1, sizeof(SOL));
  run->sol1 = calloc(1, sizeof(SOL));
  run->topo = calloc(1, sizeof(FOREST));
  CON *con = run->con;
  con->model = cfg->model;
  con->ns = cfg->ns;
  con->ischeme = cfg->ischeme;
  con->iprimtv = cfg->iprimtv;
  con->neq = cfg->neq;
  con->nprimitiv = cfg->neq; /* inputset.c:130-222 for models 1 and 3 */
  con->neq_temp = cfg->neq;
  con->turb = 0;
  con->eos = cfg->eos;
  con->i_case = cfg->i_case;
  con->ymin = cfg->ymin;
  con->dt = cfg->dt;
  con->verbose = 0;
  con->rank = 0;
  run->par->matergama[0] = cfg->gamma;
  run->par->materpinf[0] = cfg->pinf;
  run->par->matervisc[0] = cfg->visc;

  h->glob = calloc(1, sizeof(BRANCH));
  h->glob->level = 0;
  run->topo->glob = h->glob;

  h->cells = calloc((size_t)n, sizeof(BRANCH *));
  for (int64_t c = 0; c < n; ++c) {
    BRANCH *b = calloc(1, sizeof(BRANCH));
    h->cells[c] = b;
    int64_t p[3] = {ijk[c], ijk[n + c], ijk[2 * n + c]};
    b->type = 0;
    b->nlfc = 6;
    b->nlnd = 8;
    b->level = level[c];
    b->root = (int)c;
    b->part = 0;
    b->cl = make_cell_nodes(h, level[c], p);
    b->prnt = make_parent(h, level[c], p);
    CELL *cl = b->cl;
    cl->nx = calloc(6, sizeof(double));
    cl->ny = calloc(6, sizeof(double));
    cl->nz = calloc(6, sizeof(double));
    cl->nxt1 = calloc(6, sizeof(double));
    cl->nyt1 = calloc(6, sizeof(double));
    cl->nzt1 = calloc(6, sizeof(double));
    cl->nxt2 = calloc(6, sizeof(double));
    cl->nyt2 = calloc(6, sizeof(double));
    cl->nzt2 = calloc(6, sizeof(double));
    cl->Area = calloc(6, sizeof(double *));
    cl->fc = calloc(6, sizeof(FC));
    cl->Vol = vol[c];
    cl->xc = centroid[c];
    cl->yc = centroid[n + c];
    cl->zc = centroid[2 * n + c];
    for (int f = 0; f < 6; ++f) {
      cl->fc[f].nnds = 4; /* createlfc.c:20-45, hexahedron */
      cl->fc[f].type = 0;
    }
    b->neigtr = calloc(6, sizeof(BRANCH **));
    b->lfc_neigs = calloc(6, sizeof(int));
    b->neigfc = calloc(6, sizeof(int));
    b->nsfc = calloc(6, sizeof(int));
    for (int f = 0; f < 6; ++f) {
      cl->Area[f] = calloc(4, sizeof(double));
      b->neigtr[f] = calloc(4, sizeof(BRANCH *));
      const double *fr = frames + 9 * f;
      cl->nx[f] = fr[0];
      cl->ny[f] = fr[1];
      cl->nz[f] = fr[2];
      cl->nxt1[f] = fr[3];
      cl->nyt1[f] = fr[4];
      cl->nzt1[f] = fr[5];
      cl->nxt2[f] = fr[6];
      cl->nyt2[f] = fr[7];
      cl->nzt2[f] = fr[8];
    }
    if (c > 0) {
      h->cells[c - 1]->lnxt = b;
      b->lprv = h->cells[c - 1];
    }
  }
  run->topo->locl = n > 0 ? h->cells[0] : NULL;

  /* connectivity */
  for (int64_t c = 0; c < n; ++c) {
    BRANCH *b = h->cells[c];
    const int l = level[c];
    for (int f = 0; f < 6; ++f) {
      const int32_t code = nbr[(int64_t)f * n + c];
      const int a = kAxis[f];
      int64_t u[3] = {ijk[c], ijk[n + c], ijk[2 * n + c]};
      u[a] += kSign[f];
      if (code < 0 && code >= -8) { /* boundary */
        b->cl->fc[f].bc = -1 - code;
        b->lfc_neigs[f] = 1;
        b->nsfc[f] = 1;
        b->neigfc[f] = -1;
        b->neigtr[f][0] = h->glob;
        b->cl->Area[f][0] = area[(int64_t)f * n + c];
        continue;
      }
      b->cl->fc[f].bc = 0;
      b->neigfc[f] = nbr_face[(int64_t)f * n + c];
      if (code >= 0) {
        b->lfc_neigs[f] = 1;
        b->nsfc[f] = 1;
        b->cl->Area[f][0] = area[(int64_t)f * n + c];
        int64_t up[3] = {u[0], u[1], u[2]};
        if (level[code] == l - 1)
          for (int q = 0; q < 3; ++q) up[q] = fdiv2(up[q]);
        b->neigtr[f][0] = neighbour_branch(h, code, ijk, up);
      } else { /* 1:4 hanging face */
        const int64_t r = -16 - (int64_t)code;
        b->lfc_neigs[f] = 4;
        b->nsfc[f] = 4;
        for (int s = 0; s < 4; ++s) {
          const int64_t k = hang_nbr[4 * r + s];
          b->cl->Area[f][s] = hang_area[4 * r + s];
          /* fine neighbour's unwrapped position = actual + 2 * wrap shift */
          const int64_t nl = (int64_t)1 << l;
          int64_t w = u[a];
          if (w < 0 || w >= nl) w = (w + nl) % nl;
          const int64_t shift = 2 * (u[a] - w);
          int64_t up[3] = {ijk[k], ijk[n + k], ijk[2 * n + k]};
          up[a] += shift;
          b->neigtr[f][s] = neighbour_branch(h, k, ijk, up);
        }
      }
    }
  }

  memallocation(run); /* sol/sol1 + every leaf (leafallocation.c) */
  createutility(run); /* RUN scratch (createutility.c) */
  /* images share the real leaf storage */
  for (int64_t e = 0; e < h->nextra; ++e) {
    BRANCH *b = h->extra[e];
    if (b->root >= 0 && b->nlfc == 6 && b->neigtr != NULL) b->el = h->cells[b->root]->el;
  }
  return h;
}

void refh_destroy(refh *h) {
  /* The reference has no matching free routines for most of these objects
   * (leafdeallocation.c frees only part of SG); the harness lives for one
   * test and releases the branch shells only. */
  if (!h) return;
  for (int64_t e = 0; e < h->nextra; ++e) free(h->extra[e]);
  free(h->extra);
  free(h->cells);
  free(h->ijk);
  free(h);
}

void refh_set_dt(refh *h, double dt) { h->run->con->dt = dt; }

void refh_set_state(refh *h, const double *U) {
  const int neq = h->run->con->neq;
  for (int64_t c = 0; c < h->n; ++c)
    for (int v = 0; v < neq; ++v) h->cells[c]->el->S[v] = U[(int64_t)v * h->n + c];
}

/* which: 0 = S, 1 = SN, 2 = RHS, 3 = SF [6][neq][n], 4 = SG [neq+1][3][n] */
void refh_get(const refh *h, int which, double *out) {
  const int neq = h->run->con->neq;
  const int64_t n = h->n;
  for (int64_t c = 0; c < n; ++c) {
    LEAF *el = h->cells[c]->el;
    switch (which) {
      case 0:
        for (int v = 0; v < neq; ++v) out[(int64_t)v * n + c] = el->S[v];
        break;
      case 1:
        for (int v = 0; v < neq; ++v) out[(int64_t)v * n + c] = el->SN[v];
        break;
      case 2:
        for (int v = 0; v < neq; ++v) out[(int64_t)v * n + c] = el->RHS[v];
        break;
      case 3:
        for (int f = 0; f < 6; ++f)
          for (int v = 0; v < neq; ++v) out[((int64_t)f * neq + v) * n + c] = el->SF[f][v];
        break;
      case 4:
        for (int v = 0; v <= neq; ++v)
          for (int d = 0; d < 3; ++d) out[((int64_t)v * 3 + d) * n + c] = el->SG[v][d];
        break;
      default:
        break;
    }
  }
}

void refh_faceinterp(refh *h) { faceinterp(h->run); }
void refh_gradcalc(refh *h) { gradcalc(h->run); }
void refh_rhs(refh *h) { RHS(h->run); }
void refh_rk(refh *h, int irk) { RK(irk, h->run); }

/* One time step with the stage list `stages` (e.g. {1,2,3} for SSP-RK3,
 * {1,4} for SSP-RK2, {1} for forward Euler). */
void refh_step(refh *h, const int *stages, int nstages) {
  RUN *run = h->run;
  RK(0, run);
  for (int s = 0; s < nstages; ++s) {
    if (run->con->ischeme == 2) faceinterp(run);
    if (run->con->ns == 1) gradcalc(run);
    RHS(run);
    RK(stages[s], run);
  }
}

/* The reference's refinement flags (criterionsplt.c) for case i_case with
 * target level `level`; split[c] receives brch->split. */
void refh_criterion(refh *h, int i_case, int geo_adapth, int level, int32_t *split) {
  RUN *run = h->run;
  const int saved = run->con->i_case;
  run->con->i_case = i_case;
  run->con->geo_adapth = geo_adapth;
  run->con->level = level;
  criterionsplt(run);
  run->con->i_case = saved;
  for (int64_t c = 0; c < h->n; ++c) split[c] = h->cells[c]->split;
}

/* Conservation sums, conservationcalc.c:19-34 without the file output. */
void refh_conservation(const refh *h, double *sums) {
  const int neq = h->run->con->neq;
  for (int v = 0; v <= neq; ++v) sums[v] = 0.0;
  BRANCH *crnt = h->run->topo->locl;
  while (crnt != NULL) {
    for (int v = 0; v < neq; ++v) sums[v] += crnt->el->S[v] * crnt->cl->Vol;
    sums[neq] += crnt->cl->Vol;
    crnt = crnt->lnxt;
  }
}

/* The export of loop.c:50-55 in a serial run: gradcalc, then the reference's
 * Tecplot writer exportfield_linked_V3 (the halo exchange communicate_S
 * between them moves nothing on one process).  The writer walks the forest,
 * so the harness supplies one: the trees are the cells of level root_level in
 * Morton order (x bit lowest), each tree's leaves the contiguous run of the
 * leaf list under it, entered through a one-kid stand-in branch when the tree
 * has more than its root leaf.  The rest of what the writer reads: pleaves,
 * one partition with no buffer trees, octree splitting (splitmode 8), every
 * face a 4-node quadrilateral of type 0 and every neighbour angle 0 (all
 * leaves share one orientation).  The file, field_linked<tstep>prt00.dat, is
 * written to the working directory.  Returns 0, or -1 when a leaf is coarser
 * than root_level. */
static uint64_t spread3_h(uint64_t x) {
  uint64_t r = 0;
  for (int b = 0; b < 21; ++b) r |= ((x >> b) & 1ull) << (3 * b);
  return r;
}

int refh_export(refh *h, int root_level, int tstep) {
  RUN *run = h->run;
  const int64_t n = h->n;
  for (int64_t c = 0; c < n; ++c)
    if (h->cells[c]->level < root_level) return -1;
  const int64_t ntrees = (int64_t)1 << (3 * root_level);
  TREE **drys = calloc((size_t)ntrees, sizeof(TREE *));
  BRANCH **stubs = calloc((size_t)ntrees, sizeof(BRANCH *));
  for (int64_t c = 0; c < n; ++c) {
    BRANCH *b = h->cells[c];
    const int sh = b->level - root_level;
    const uint64_t t = spread3_h((uint64_t)(h->ijk[c] >> sh)) | (spread3_h((uint64_t)(h->ijk[n + c] >> sh)) << 1) |
                       (spread3_h((uint64_t)(h->ijk[2 * n + c] >> sh)) << 2);
    b->root = (int)t;
    if (!drys[t]) {
      drys[t] = calloc(1, sizeof(TREE));
      drys[t]->part = 0;
      drys[t]->brch = b;
    } else if (!stubs[t]) {
      BRANCH *first = drys[t]->brch;
      stubs[t] = calloc(1, sizeof(BRANCH));
      stubs[t]->nkids = 1;
      stubs[t]->kids = calloc(1, sizeof(BRANCH *));
      stubs[t]->kids[0] = first;
      stubs[t]->root = (int)t;
      drys[t]->brch = stubs[t];
    }
    if (!b->neigag) b->neigag = calloc(6, sizeof(int));
    for (int f = 0; f < 6; ++f) {
      b->cl->fc[f].nnds = 4;
      b->cl->fc[f].type = 0;
    }
  }
  FOREST *topo = run->topo;
  topo->ntrees = (int)ntrees;
  topo->drys = drys;
  topo->pleaves = (int)n;
  int *nbuff = calloc(1, sizeof(int));
  topo->nbuff = nbuff;
  run->con->size = 1;
  run->con->rank = 0;
  run->con->splitmode = 8;
  run->con->tstep = tstep;

  gradcalc(run);
  exportfield_linked_V3(run);

  for (int64_t t = 0; t < ntrees; ++t) {
    if (stubs[t]) {
      free(stubs[t]->kids);
      free(stubs[t]);
    }
    free(drys[t]);
  }
  free(stubs);
  free(drys);
  free(nbuff);
  topo->drys = NULL;
  topo->nbuff = NULL;
  topo->ntrees = 0;
  return 0;
}

/* The reference's own geometry of every leaf from the harness's node
 * coordinates: cell volume (volmproperties), face and sub-face areas
 * (areaproperties; a 1:4 face's four areas come from the fine neighbours'
 * faces, in neigtr order) and the per-face frames n, t1, t2
 * (normalvectorcalc, tagvectorcalc), all from meshproperties.c, normalvector.c
 * and tagvector.c.  vol [n], area [6][4][n] (zero where a face has fewer
 * sub-faces), frames [6][9][n].  The leaves' own geometry fields are
 * overwritten with these values. */
void refh_geometry(refh *h, double *vol, double *area, double *frames) {
  RUN *run = h->run;
  const int64_t n = h->n;
  for (int64_t c = 0; c < n; ++c) {
    BRANCH *b = h->cells[c];
    areaproperties(b, run);
    volmproperties(0, b, run);
    normalvectorcalc(run, b);
    tagvectorcalc(run, b);
    CELL *cl = b->cl;
    vol[c] = cl->Vol;
    for (int f = 0; f < 6; ++f) {
      for (int s = 0; s < 4; ++s) area[((int64_t)f * 4 + s) * n + c] = s < b->nsfc[f] ? cl->Area[f][s] : 0.0;
      const double fr[9] = {cl->nx[f], cl->ny[f], cl->nz[f], cl->nxt1[f], cl->nyt1[f],
                            cl->nzt1[f], cl->nxt2[f], cl->nyt2[f], cl->nzt2[f]};
      for (int k = 0; k < 9; ++k) frames[((int64_t)f * 9 + k) * n + c] = fr[k];
    }
  }
}
