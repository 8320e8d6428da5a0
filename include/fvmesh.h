/*
 * fvmesh.h -- host-side octree mesh builder and flattener (C ABI).
 *
 * The reference keeps its forest of octrees on the host (split.c, merge.c,
 * elconn.c, rebuildconn.c) and walks the leaf list `run->topo->locl` on every
 * residual evaluation.  This library is the synthetic stand-in for that host:
 * it builds an axis-aligned, 2:1 face-balanced octree over a box, orders the
 * leaves along a Morton curve and flattens leaves and faces -- including the
 * 1:4 hanging faces -- into the structure-of-arrays tables that
 * libfvgpu uploads once per adaptation (fvgpu.h, fvgpu_mesh_soa).
 *
 * Conventions taken from the reference's hexahedron tables (operatetp.c):
 *   local node n has bit0 = +x, bit1 = +y, bit2 = +z
 *   face f: 0 = -y, 1 = +x, 2 = +y, 3 = -x, 4 = -z, 5 = +z
 *   opposite face (fcopp, operatetp.c:481-490): 0<->2, 1<->3, 4<->5
 * MUSCL stencil distances follow distance.c:3-148 term by term.
 *
 * Every function returns 0 on success and a negative FVMESH_ERR_* code on
 * failure; fvmesh_last_error() returns a message for the calling thread.
 */
#ifndef FVMESH_H
#define FVMESH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FVMESH_ERR_ARG      (-1)   /* bad argument */
#define FVMESH_ERR_BALANCE  (-2)   /* 2:1 face balance violated */
#define FVMESH_ERR_LEVEL    (-3)   /* level outside [1, FVMESH_MAX_LEVEL] */
#define FVMESH_ERR_NOMEM    (-4)

#define FVMESH_MAX_LEVEL 18

/* Boundary codes carried in fvmesh face tables (bc.c:19-49). */
#define FVMESH_BC_NONE        0
#define FVMESH_BC_INFLOW      1
#define FVMESH_BC_TRANSMISSIVE 2
#define FVMESH_BC_REFLECTIVE  3
#define FVMESH_BC_NOSLIP      4

/* Neighbour code stored per (face, cell):
 *   code >= 0            : the single neighbour cell (same level or one coarser)
 *   -8 <= code <= -1     : boundary face with bc = -1 - code
 *   code <= FVMESH_HANG0 : 1:4 hanging face, record index = FVMESH_HANG0 - code */
#define FVMESH_HANG0 (-16)

typedef struct fvmesh fvmesh;

/* Flattened tables. The caller allocates every array with the sizes given by
 * fvmesh_sizes() and passes the pointers; fvmesh_flatten() fills them.
 * Layout is structure-of-arrays: [face][cell] means index f*ncells + c. */
typedef struct fvmesh_tables {
  int32_t *level;      /* [ncells] octree level (root = 0) */
  int32_t *ijk;        /* [3][ncells] integer position at the cell's level */
  int32_t *nbr;        /* [6][ncells] neighbour code, see above */
  int32_t *nbr_face;   /* [6][ncells] neighbour's face index (neigfc), -1 at boundaries */
  double  *area;       /* [6][ncells] face area (single-neighbour and boundary faces) */
  double  *dcf;        /* [6][ncells] centroid-to-face distance, distance.c */
  double  *dcc;        /* [6][ncells] centroid-to-centroid distance, distance.c */
  double  *vol;        /* [ncells] */
  double  *centroid;   /* [3][ncells] */
  int32_t *hang_nbr;   /* [nhang][4] fine neighbours of a 1:4 face; neighbour s
                          holds the face's node s, fcnd2elnd(f, s), as a corner
                          (the reference's order, elconnfin.c:42-45) */
  double  *hang_area;  /* [nhang][4] sub-face areas */
  int32_t *hang_cell;  /* [nhang] owning (coarse) cell */
  int32_t *hang_face;  /* [nhang] owning face index */
  double  *frames;     /* [6][9] per face index: n(3), t1(3), t2(3) */
} fvmesh_tables;

/* Box [lo, lo+len] refined uniformly to base_level.  periodic[a] != 0 wraps
 * axis a; side_bc[f] is the boundary code of the domain side facing the same
 * way as face f (ignored on periodic axes). */
int fvmesh_create_uniform(const double lo[3], const double len[3], int base_level,
                          const int periodic[3], const int side_bc[6], fvmesh **out);
void fvmesh_destroy(fvmesh *m);

/* Number of leaves and of 1:4 hanging-face records. */
int fvmesh_sizes(const fvmesh *m, int64_t *ncells, int64_t *nhang);

/* Leaf levels and centroids (centroids as distance.c forms them: node average). */
int fvmesh_leaves(const fvmesh *m, int32_t *level, double *centroid /*[3][n]*/);

/* Leaf levels and lattice positions (ijk[a * n + c]: the leaf's index along
 * axis a at its own level), in Morton order: the leaf list fvgpu_upload_leaves
 * takes, without flattening on the host. */
int fvmesh_leaf_cells(const fvmesh *m, int32_t *level, int32_t *ijk /*[3][n]*/);

/* Refine every leaf whose flag is nonzero (up to max_level), then refine more
 * leaves until every face sees at most one level of difference.  Leaves are
 * re-sorted along the Morton curve. */
int fvmesh_refine(fvmesh *m, const uint8_t *flags, int max_level);

/* One adaptation pass (meshadaptation.c:23-58) from per-leaf target levels
 * split[ncells] (criterionsplt.c; fvgpu_criterion gives them): each leaf
 * moves at most one level toward its target, as criterionsmth.c smooths it;
 * 8 sibling leaves that all ask for a coarser level merge (refineh_1.c:30-62)
 * unless the parent would sit next to a finer face neighbour; 2:1 face
 * balance follows.  Levels stay within [min_level, max_level].  Records the
 * state-transfer plan that fvmesh_transfer applies. */
int fvmesh_adapt(fvmesh *m, const int32_t *split, int min_level, int max_level);

/* State transfer of the last fvmesh_adapt: S_old [neq][n_old] on the leaves
 * before it -> S_new [neq][ncells] on the current leaves.  A split leaf's
 * children take its state (split.c:493); a merged parent takes the sum of its
 * 8 children's states each divided by 8, in child order (merge.c:93-101). */
int fvmesh_transfer(const fvmesh *m, int neq, int64_t n_old, const double *S_old, double *S_new);

/* Fill the flattened tables (caller-allocated, sizes from fvmesh_sizes). */
int fvmesh_flatten(const fvmesh *m, const fvmesh_tables *t);

/* Node coordinates as the reference stores them in CELL.nd (8 nodes, local
 * numbering above) for the cell at (level, i, j, k); i, j, k may lie outside
 * the box (periodic images).  Used by the reference harness. */
int fvmesh_cell_nodes(const fvmesh *m, int level, int i, int j, int k, double xyz[8][3]);

/* Domain description. */
int fvmesh_domain(const fvmesh *m, double lo[3], double len[3], int periodic[3], int side_bc[6]);

const char *fvmesh_last_error(void);

/* Tecplot export, exportfield_linked_V3.c:19-572 (called by loop.c:50-55
 * after gradcalc).  Writes `path` with the reference's bytes: a " VARIABLES"
 * line, a ZONE line (FEPOINT, BRICK), one point per node link (x y z, iel,
 * part, then the link means of S[0..neq), P and |grad| of rho, u, v and p),
 * then 8 one-based link numbers per leaf.  The leaf field comes from the
 * caller (e.g. downloaded from libfvgpu): S [neq][n] and SG [neq+1][3][n]
 * (fvgpu_gradcalc's layout; NULL prints zero gradients, as leaves that were
 * never differentiated hold, leafallocation.c:36-40).  Tables as
 * fvmesh_flatten fills them; lo/len the box.  Trees of the forest (the "iel"
 * column) are the cells of level root_level, numbered along the Morton
 * curve; no leaf may be coarser than root_level. */
typedef struct fvmesh_tecplot {
  int model;       /* 1 ideal gas (neq 5), 2 barotropic (neq 4), 3 mixture (neq 5) */
  int neq;
  int root_level;
  int pad;
  double gamma;    /* matergama[0] */
  double pinf;     /* materpinf[0] */
} fvmesh_tecplot;

int fvmesh_export_tecplot(const fvmesh_tecplot *cfg, int64_t ncells, const int32_t *level,
                          const int32_t *ijk, const int32_t *nbr, const int32_t *hang_nbr,
                          int64_t nhang, const double lo[3], const double len[3],
                          const double *S, const double *SG, const char *path);
const char *fvmesh_export_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
