/*
 * parmetis.h -- ParMETIS_V3_AdaptiveRepart as the reference calls it
 * (repartition_parmetis.c:226) for a single process: every local vertex stays
 * on part 0 (the only rank).  Definition in fvcompat.c.
 */
#ifndef FVCOMPAT_PARMETIS_H
#define FVCOMPAT_PARMETIS_H
#include "metis.h"
#include "mpi.h"

#ifdef __cplusplus
extern "C" {
#endif

int ParMETIS_V3_AdaptiveRepart(idx_t *vtxdist, idx_t *xadj, idx_t *adjncy, idx_t *vwgt, idx_t *vsize,
                               idx_t *adjwgt, idx_t *wgtflag, idx_t *numflag, idx_t *ncon, idx_t *nparts,
                               real_t *tpwgts, real_t *ubvec, real_t *ipc2redist, idx_t *options, idx_t *edgecut,
                               idx_t *part, MPI_Comm *comm);

#ifdef __cplusplus
}
#endif
#endif
