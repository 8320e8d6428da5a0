// Device-side flattening of a Morton-sorted leaf list (fv_flatten.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fv {

// the box and its sides (fvmesh_create_uniform's arguments)
struct LeafGeom {
  double lo[3], len[3];
  int periodic[3];
  int side_bc[6];
};

// device outputs, layouts of fvgpu_mesh_soa
struct DevTables {
  int32_t *nbr, *nbr_face, *hang_nbr, *level;
  double *area, *dcf, *dcc, *vol, *hang_area;
};

// Pass 1: Morton keys (checked strictly increasing), 1:4 faces per cell and
// their exclusive scan (the first record number of each cell); *nhang (device)
// receives the total.  err (device) gets code << 40 | cell: 1 = level or
// position out of range, 2 = leaves not in Morton order.
cudaError_t flatten_count(const LeafGeom &g, int64_t n, const int32_t *level, const int32_t *ijk, uint64_t *keys,
                          int32_t *counts, int64_t *tile_sums, int64_t *nhang, unsigned long long *err,
                          cudaStream_t st);
// Pass 2: the tables (err code 3: a face sees more than one level).
cudaError_t flatten_tables(const LeafGeom &g, int64_t n, const int32_t *level, const int32_t *ijk,
                           const uint64_t *keys, const int32_t *offsets, const DevTables &t, unsigned long long *err,
                           cudaStream_t st);

}  // namespace fv
