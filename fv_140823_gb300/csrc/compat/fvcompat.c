/*
 * fvcompat.c -- what the reference's host program (main.c:16-187 and the
 * files it links) needs beyond its own sources to build and run as one
 * process: serial MPI, METIS / ParMETIS that put everything on part 0, a
 * PETSc start-up that does nothing, and the host routines the reference
 * declares but does not ship (strdata.h:629, 709-710; bc.c:38,42):
 *
 *   cellallocation / celldeallocation  the CELL of a branch;
 *   brchconn                            neighbour links of a split's kids;
 *   bc_reflective / bc_wall             slip and no-slip wall ghost states.
 *
 * Built against the reference's strdata.h with the headers in include/ of
 * this directory in front of the system's.  With the drop-in shim
 * (csrc/shim/fvshim.c) and libfvgpu the program's residual path runs on the
 * GPU; with fvcompat_cpu.c it runs on its own C code.
 */
#include "strdata.h"

#include <stdint.h>
#include <time.h>

/* ---- serial MPI ---------------------------------------------------------- */

static size_t type_size(MPI_Datatype dt) {
  switch (dt) {
    case MPI_CHAR: return 1;
    case MPI_INT: return sizeof(int);
    case MPI_FLOAT: return sizeof(float);
    case MPI_LONG: return sizeof(long);
    case MPI_DOUBLE: return sizeof(double);
    default: return 0;
  }
}

static void mpi_fail(const char *what, int tag) {
  fprintf(stderr, "fvcompat: %s (tag %d): a one-process run cannot satisfy it\n", what, tag);
  exit(1);
}

/* messages a rank sent to itself, oldest first */
typedef struct fvc_msg {
  int tag;
  size_t bytes;
  struct fvc_msg *next;
  unsigned char data[];
} fvc_msg;
static fvc_msg *g_head = NULL, *g_tail = NULL;

/* receives posted before their message: request r refers to g_pend[r - 1] */
typedef struct {
  void *buf;
  size_t bytes;
  int tag, live;
} fvc_pending;
static fvc_pending *g_pend = NULL;
static int g_npend = 0, g_cappend = 0;

static int take(void *buf, size_t bytes, int tag, MPI_Status *st) {
  fvc_msg *prev = NULL;
  for (fvc_msg *m = g_head; m; prev = m, m = m->next) {
    if (m->tag != tag) continue;
    memcpy(buf, m->data, m->bytes < bytes ? m->bytes : bytes);
    if (st) {
      st->MPI_SOURCE = 0;
      st->MPI_TAG = tag;
      st->MPI_ERROR = MPI_SUCCESS;
      st->count_bytes = (int)(m->bytes < bytes ? m->bytes : bytes);
    }
    if (prev) prev->next = m->next; else g_head = m->next;
    if (g_tail == m) g_tail = prev;
    free(m);
    return 1;
  }
  return 0;
}

int MPI_Init(int *argc, char ***argv) {
  (void)argc, (void)argv;
  return MPI_SUCCESS;
}
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm comm, int *rank) {
  (void)comm;
  *rank = 0;
  return MPI_SUCCESS;
}
int MPI_Comm_size(MPI_Comm comm, int *size) {
  (void)comm;
  *size = 1;
  return MPI_SUCCESS;
}
int MPI_Barrier(MPI_Comm comm) {
  (void)comm;
  return MPI_SUCCESS;
}
double MPI_Wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype dt, MPI_Op op, MPI_Comm comm) {
  (void)op, (void)comm;
  memmove(r, s, (size_t)n * type_size(dt));
  return MPI_SUCCESS;
}
int MPI_Bcast(void *buf, int n, MPI_Datatype dt, int root, MPI_Comm comm) {
  (void)buf, (void)n, (void)dt, (void)comm;
  return root == 0 ? MPI_SUCCESS : MPI_ERR_OTHER;
}
int MPI_Send(const void *buf, int n, MPI_Datatype dt, int dest, int tag, MPI_Comm comm) {
  (void)comm;
  if (dest != 0) mpi_fail("MPI_Send to a rank other than 0", tag);
  const size_t bytes = (size_t)n * type_size(dt);
  /* a receive posted earlier takes the message at once */
  for (int r = 0; r < g_npend; ++r) {
    if (g_pend[r].live && g_pend[r].tag == tag) {
      memcpy(g_pend[r].buf, buf, bytes < g_pend[r].bytes ? bytes : g_pend[r].bytes);
      g_pend[r].live = 0;
      return MPI_SUCCESS;
    }
  }
  fvc_msg *m = malloc(sizeof(fvc_msg) + bytes);
  m->tag = tag;
  m->bytes = bytes;
  m->next = NULL;
  memcpy(m->data, buf, bytes);
  if (g_tail) g_tail->next = m; else g_head = m;
  g_tail = m;
  return MPI_SUCCESS;
}
int MPI_Recv(void *buf, int n, MPI_Datatype dt, int source, int tag, MPI_Comm comm, MPI_Status *st) {
  (void)comm;
  if (source != 0 || !take(buf, (size_t)n * type_size(dt), tag, st)) mpi_fail("MPI_Recv without a matching send", tag);
  return MPI_SUCCESS;
}
int MPI_Isend(const void *buf, int n, MPI_Datatype dt, int dest, int tag, MPI_Comm comm, MPI_Request *req) {
  *req = MPI_REQUEST_NULL;
  return MPI_Send(buf, n, dt, dest, tag, comm);
}
int MPI_Irecv(void *buf, int n, MPI_Datatype dt, int source, int tag, MPI_Comm comm, MPI_Request *req) {
  (void)comm;
  if (source != 0) mpi_fail("MPI_Irecv from a rank other than 0", tag);
  const size_t bytes = (size_t)n * type_size(dt);
  if (take(buf, bytes, tag, NULL)) {
    *req = MPI_REQUEST_NULL;
    return MPI_SUCCESS;
  }
  if (g_npend == g_cappend) {
    g_cappend = g_cappend ? 2 * g_cappend : 16;
    g_pend = realloc(g_pend, (size_t)g_cappend * sizeof(fvc_pending));
  }
  g_pend[g_npend] = (fvc_pending){buf, bytes, tag, 1};
  *req = ++g_npend;
  return MPI_SUCCESS;
}
int MPI_Wait(MPI_Request *req, MPI_Status *st) {
  if (*req != MPI_REQUEST_NULL) {
    fvc_pending *p = &g_pend[*req - 1];
    if (p->live) mpi_fail("MPI_Wait on a receive no send matched", p->tag);
    *req = MPI_REQUEST_NULL;
  }
  if (st) st->MPI_ERROR = MPI_SUCCESS;
  return MPI_SUCCESS;
}

/* ---- METIS / ParMETIS / PETSc --------------------------------------------- */

int METIS_PartGraphRecursive(idx_t *nvtxs, idx_t *ncon, idx_t *xadj, idx_t *adjncy, idx_t *vwgt, idx_t *vsize,
                             idx_t *adjwgt, idx_t *nparts, real_t *tpwgts, real_t *ubvec, idx_t *options,
                             idx_t *objval, idx_t *part) {
  (void)ncon, (void)xadj, (void)adjncy, (void)vwgt, (void)vsize, (void)adjwgt, (void)nparts, (void)tpwgts,
      (void)ubvec, (void)options;
  for (idx_t i = 0; i < *nvtxs; ++i) part[i] = 0;
  if (objval) *objval = 0;
  return METIS_OK;
}
int METIS_PartGraphKway(idx_t *nvtxs, idx_t *ncon, idx_t *xadj, idx_t *adjncy, idx_t *vwgt, idx_t *vsize,
                        idx_t *adjwgt, idx_t *nparts, real_t *tpwgts, real_t *ubvec, idx_t *options, idx_t *objval,
                        idx_t *part) {
  return METIS_PartGraphRecursive(nvtxs, ncon, xadj, adjncy, vwgt, vsize, adjwgt, nparts, tpwgts, ubvec, options,
                                  objval, part);
}
int ParMETIS_V3_AdaptiveRepart(idx_t *vtxdist, idx_t *xadj, idx_t *adjncy, idx_t *vwgt, idx_t *vsize,
                               idx_t *adjwgt, idx_t *wgtflag, idx_t *numflag, idx_t *ncon, idx_t *nparts,
                               real_t *tpwgts, real_t *ubvec, real_t *ipc2redist, idx_t *options, idx_t *edgecut,
                               idx_t *part, MPI_Comm *comm) {
  (void)xadj, (void)adjncy, (void)vwgt, (void)vsize, (void)adjwgt, (void)wgtflag, (void)numflag, (void)ncon,
      (void)nparts, (void)tpwgts, (void)ubvec, (void)ipc2redist, (void)options, (void)comm;
  for (idx_t i = 0; i < vtxdist[1] - vtxdist[0]; ++i) part[i] = 0;
  if (edgecut) *edgecut = 0;
  return METIS_OK;
}
PetscErrorCode PetscInitialize(int *argc, char ***args, const char *file, const char *help) {
  (void)argc, (void)args, (void)file, (void)help;
  return 0;
}
PetscErrorCode PetscFinalize(void) { return 0; }

/* ---- host routines the reference declares without a definition ----------- */

/* The CELL of a branch: node coordinates, face records, per-face frames and
 * up to four sub-face areas per face (the most a face of a 2:1 balanced
 * octree has, residual_faces_AMR.c:25), all zero. */
void cellallocation(struct BRANCH *brch) {
  const int nf = brch->nlfc > 0 ? brch->nlfc : 1;
  const int nn = brch->nlnd > 0 ? brch->nlnd : 1;
  CELL *cl = calloc(1, sizeof(CELL));
  cl->nd = calloc((size_t)nn, sizeof(ND));
  cl->fc = calloc((size_t)nf, sizeof(FC));
  double **frames[9] = {&cl->nx, &cl->ny, &cl->nz, &cl->nxt1, &cl->nyt1, &cl->nzt1, &cl->nxt2, &cl->nyt2, &cl->nzt2};
  for (int k = 0; k < 9; ++k) *frames[k] = calloc((size_t)nf, sizeof(double));
  cl->Area = calloc((size_t)nf, sizeof(double *));
  for (int f = 0; f < nf; ++f) cl->Area[f] = calloc(4, sizeof(double));
  brch->cl = cl;
}

void celldeallocation(struct BRANCH *crnt) {
  CELL *cl = crnt ? crnt->cl : NULL;
  if (!cl) return;
  const int nf = crnt->nlfc > 0 ? crnt->nlfc : 1;
  for (int f = 0; f < nf; ++f) free(cl->Area[f]);
  free(cl->Area);
  free(cl->nx), free(cl->ny), free(cl->nz);
  free(cl->nxt1), free(cl->nyt1), free(cl->nzt1);
  free(cl->nxt2), free(cl->nyt2), free(cl->nzt2);
  free(cl->fc);
  free(cl->nd);
  free(cl);
  crnt->cl = NULL;
}

/* Face f's element nodes in face-node order, fcnd2elnd (operatetp.c:113-147)
 * for a hexahedron.  They fix what "x", "y" and "z" are for a hex of any
 * numbering the reference accepts: node n has its x bit set when it lies on
 * face 1, y on face 2 and z on face 5. */
static const int kHexFaceNode[6][4] = {{0, 1, 5, 4}, {3, 7, 5, 1}, {2, 6, 7, 3}, {2, 0, 4, 6}, {2, 3, 1, 0}, {6, 4, 5, 7}};

static int on_face(int node, int f) {
  for (int s = 0; s < 4; ++s)
    if (kHexFaceNode[f][s] == node) return 1;
  return 0;
}

/* Neighbour links of the kids of a branch that split.c has just split (its
 * last call, split.c:513).  Kid k sits at the parent's corner node k
 * (split.c:110-123).  Across face f, kid k either meets a sibling -- the kid
 * at the corner that shares the edge through node k normal to face f, whose
 * face toward k is the opposite face (fcopp, operatetp.c:481-490) at angle 0
 * since siblings share one numbering -- or lies on the parent's face f, in
 * which case its link is the parent itself: elconn.c:31-55 then walks up
 * from the parent through its own keen[f] to the branch across.  The links
 * of the parent's neighbours and of the leaf list are rebuilt by
 * restructtopo (rebuildprox / rebuildconn) before any face loop runs. */
void brchconn(BRANCH *brch) {
  if (brch->type != 0 || brch->nkids != 8) {
    fprintf(stderr, "fvcompat: brchconn supports hexahedra split into 8 (type %d, %d kids)\n", brch->type,
            brch->nkids);
    exit(1);
  }
  static const int kOppFace[6] = {2, 3, 0, 1, 5, 4};
  static const int kAxisFace[3] = {1, 2, 5}; /* the face that carries each axis bit */
  for (int k = 0; k < 8; ++k) {
    BRANCH *kid = brch->kids[k];
    for (int f = 0; f < 6; ++f) {
      if (on_face(k, f)) {
        kid->keen[f] = brch;
        kid->keenfc[f] = f;
        kid->keenfcangle[f] = 0;
        continue;
      }
      /* the sibling across face f: node k moved along the axis normal to f */
      int sib = -1;
      for (int a = 0; a < 3; ++a) {
        const int g = kAxisFace[a];
        if (g != f && kOppFace[g] != f) continue;
        for (int m = 0; m < 8; ++m) {
          int same = 1;
          for (int b = 0; b < 3; ++b)
            if (b != a && on_face(m, kAxisFace[b]) != on_face(k, kAxisFace[b])) same = 0;
          if (same && m != k) sib = m;
        }
      }
      kid->keen[f] = brch->kids[sib];
      kid->keenfc[f] = kOppFace[f];
      kid->keenfcangle[f] = 0;
    }
  }
}

/* Ghost state of a slip wall on run->sol1 (bc.c:38): the normal component of
 * velocity and momentum mirrored across face f's outward normal; density,
 * energy, pressure and sound speed kept.  No reference code exists for it;
 * libfvgpu applies the same ghost. */
void bc_reflective(struct BRANCH *crnt, int f, RUN *run) {
  SOL *g = run->sol1;
  const double nx = crnt->cl->nx[f], ny = crnt->cl->ny[f], nz = crnt->cl->nz[f];
  const double un = (g->u * nx + g->v * ny) + g->w * nz;
  g->u = g->u - 2.0 * un * nx;
  g->v = g->v - 2.0 * un * ny;
  g->w = g->w - 2.0 * un * nz;
  const double mn = (g->vec[1] * nx + g->vec[2] * ny) + g->vec[3] * nz;
  g->vec[1] = g->vec[1] - 2.0 * mn * nx;
  g->vec[2] = g->vec[2] - 2.0 * mn * ny;
  g->vec[3] = g->vec[3] - 2.0 * mn * nz;
}

/* Ghost state of a no-slip wall on run->sol1 (bc.c:42): velocity and
 * momentum reversed, the rest kept. */
void bc_wall(struct BRANCH *crnt, int f, struct RUN *run) {
  (void)crnt, (void)f;
  SOL *g = run->sol1;
  g->u = -g->u;
  g->v = -g->v;
  g->w = -g->w;
  g->vec[1] = -g->vec[1];
  g->vec[2] = -g->vec[2];
  g->vec[3] = -g->vec[3];
}
