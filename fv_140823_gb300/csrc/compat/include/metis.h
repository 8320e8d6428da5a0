/*
 * metis.h -- the METIS 5 calls the reference makes (partitiondrys.c:61,
 * repartition.c:117) for a single process: every vertex goes to part 0.
 * 32-bit indices and reals, METIS's default widths.  Definitions in
 * fvcompat.c.
 */
#ifndef FVCOMPAT_METIS_H
#define FVCOMPAT_METIS_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t idx_t;
typedef float real_t;
#define METIS_OK 1
#define METIS_NOPTIONS 40

int METIS_PartGraphRecursive(idx_t *nvtxs, idx_t *ncon, idx_t *xadj, idx_t *adjncy, idx_t *vwgt, idx_t *vsize,
                             idx_t *adjwgt, idx_t *nparts, real_t *tpwgts, real_t *ubvec, idx_t *options,
                             idx_t *objval, idx_t *part);
int METIS_PartGraphKway(idx_t *nvtxs, idx_t *ncon, idx_t *xadj, idx_t *adjncy, idx_t *vwgt, idx_t *vsize,
                        idx_t *adjwgt, idx_t *nparts, real_t *tpwgts, real_t *ubvec, idx_t *options,
                        idx_t *objval, idx_t *part);

#ifdef __cplusplus
}
#endif
#endif
