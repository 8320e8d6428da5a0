// fvbuild: -fmad=false
//
// Device-side flattening: the SoA tables of fvgpu_mesh_soa built on the GPU
// from the Morton-sorted leaf list (level and integer position of every
// leaf), with the host builder's arithmetic (csrc/host/fvmesh.cpp,
// fvmesh_flatten: distance.c's centroid and distance rules, the same face
// numbering and 1:4 records in cell-then-face order), so both produce the
// same tables bit for bit.  The host keeps its octree; after an adaptation
// it uploads 16 bytes per leaf instead of flattening on the CPU.
//
// Passes: Morton keys (and a check that the list is sorted), hanging-face
// counts per cell, an exclusive scan of the counts (record numbers), and the
// tables.  Leaves are found by binary search of the sorted keys.
#include <cstdint>

#include "fv_flatten.cuh"

namespace fv {

namespace {

constexpr int kMaxLevel = 18;  // FVMESH_MAX_LEVEL
constexpr int kBlock = 256;
// face f -> axis, outward sign, opposite face (operatetp.c:481-490)
__host__ __device__ constexpr int axis_of(int f) { return (f == 1 || f == 3) ? 0 : ((f == 0 || f == 2) ? 1 : 2); }
__host__ __device__ constexpr int sign_of(int f) { return (f == 1 || f == 2 || f == 5) ? 1 : -1; }
__host__ __device__ constexpr int opp_of(int f) { return f ^ (f < 4 ? 2 : 1); }
// element node of face f at face node s, fcnd2elnd (operatetp.c:113-147, type
// 0); node n sits at offset (n & 1, n >> 1 & 1, n >> 2 & 1) in (x, y, z)
__host__ __device__ constexpr int face_node(int f, int s) {
  return int((f == 0 ? 0x4510u : f == 1 ? 0x1573u : f == 2 ? 0x3762u : f == 3 ? 0x6402u : f == 4 ? 0x0132u : 0x7546u) >>
             (4 * s)) & 0xf;
}

__device__ __forceinline__ uint64_t spread3(uint64_t x) {
  x &= 0x1fffff;
  x = (x | x << 32) & 0x1f00000000ffffULL;
  x = (x | x << 16) & 0x1f0000ff0000ffULL;
  x = (x | x << 8) & 0x100f00f00f00f00fULL;
  x = (x | x << 4) & 0x10c30c30c30c30c3ULL;
  x = (x | x << 2) & 0x1249249249249249ULL;
  return x;
}

__device__ __forceinline__ uint64_t morton(int level, int64_t i, int64_t j, int64_t k) {
  const int sh = kMaxLevel - level;
  return spread3(uint64_t(i) << sh) | (spread3(uint64_t(j) << sh) << 1) | (spread3(uint64_t(k) << sh) << 2);
}

__device__ __forceinline__ int64_t floordiv2(int64_t a) { return a >= 0 ? a / 2 : -((-a + 1) / 2); }

struct View {
  LeafGeom g;
  int64_t n;
  const int32_t *level, *ijk;
  const uint64_t *keys;

  __device__ double h(int level, int a) const { return ldexp(g.len[a], -level); }
  __device__ double coord(int level, int a, int64_t I) const { return g.lo[a] + double(I) * h(level, a); }
  // areaproperties (meshproperties.c:29-63): face f's two triangles (face
  // nodes 0,1,2 and 0,2,3), half the norm of each cross product, summed
  __device__ double face_area(int level, const int64_t p[3], int f) const {
    double nd[4][3];
    for (int s = 0; s < 4; ++s)
      for (int a = 0; a < 3; ++a) nd[s][a] = coord(level, a, p[a] + ((face_node(f, s) >> a) & 1));
    double area = 0.0;
    for (int it = 0; it < 2; ++it) {
      const double dx1 = nd[1 + it][0] - nd[0][0], dx2 = nd[2 + it][0] - nd[0][0];
      const double dy1 = nd[1 + it][1] - nd[0][1], dy2 = nd[2 + it][1] - nd[0][1];
      const double dz1 = nd[1 + it][2] - nd[0][2], dz2 = nd[2 + it][2] - nd[0][2];
      const double cx = dy1 * dz2 - dz1 * dy2, cy = dz1 * dx2 - dx1 * dz2, cz = dx1 * dy2 - dy1 * dx2;
      area += fabs(0.5 * sqrt(cx * cx + cy * cy + cz * cz));
    }
    return area;
  }
  // volmproperties (meshproperties.c:66-111), hexahedron: six tetrahedra on
  // node 0, triple product over 6.0, summed in order (no contraction: this
  // file builds with -fmad=false)
  __device__ double volume(int level, const int64_t p[3]) const {
    const int tet[6][3] = {{1, 3, 5}, {5, 3, 7}, {5, 7, 4}, {3, 2, 7}, {7, 2, 6}, {7, 6, 4}};
    double o[3];
    for (int a = 0; a < 3; ++a) o[a] = coord(level, a, p[a]);
    double vol = 0.0;
    for (int it = 0; it < 6; ++it) {
      double d[3][3];
      for (int in = 0; in < 3; ++in)
        for (int a = 0; a < 3; ++a) d[in][a] = coord(level, a, p[a] + ((tet[it][in] >> a) & 1)) - o[a];
      const double c0 = d[0][1] * d[1][2] - d[0][2] * d[1][1];
      const double c1 = d[0][2] * d[1][0] - d[0][0] * d[1][2];
      const double c2 = d[0][0] * d[1][1] - d[0][1] * d[1][0];
      vol += (c0 * d[2][0] + c1 * d[2][1] + c2 * d[2][2]) / 6.0;
    }
    return vol;
  }
  __device__ void centroid(int level, const int64_t p[3], double c[3]) const {
    for (int a = 0; a < 3; ++a) {
      const double lo = coord(level, a, p[a]), hi = coord(level, a, p[a] + 1);
      double s = 0.0;
      for (int nd = 0; nd < 8; ++nd) s += ((nd >> a) & 1 ? hi : lo) / 8.0;
      c[a] = s;
    }
  }
  // leaf at exactly (level, p), or -1
  __device__ int64_t find(int level, const int64_t p[3]) const {
    if (level < 0 || level > kMaxLevel) return -1;
    const int64_t m = int64_t(1) << level;
    for (int a = 0; a < 3; ++a)
      if (p[a] < 0 || p[a] >= m) return -1;
    const uint64_t key = morton(level, p[0], p[1], p[2]);
    int64_t lo = 0, hi = n - 1;
    while (lo <= hi) {
      const int64_t mid = (lo + hi) >> 1;
      const uint64_t k = keys[mid];
      if (k == key) return level == this->level[mid] ? mid : -1;
      if (k < key) lo = mid + 1; else hi = mid - 1;
    }
    return -1;
  }
  __device__ bool neighbour_pos(int level, const int64_t p[3], int f, int64_t w[3], int64_t u[3]) const {
    const int a = axis_of(f);
    const int64_t m = int64_t(1) << level;
    for (int b = 0; b < 3; ++b) u[b] = w[b] = p[b];
    u[a] += sign_of(f);
    w[a] = u[a];
    if (w[a] < 0 || w[a] >= m) {
      if (!g.periodic[a]) return false;
      w[a] = (w[a] + m) % m;
    }
    return true;
  }
  __device__ void pos(int64_t c, int64_t p[3]) const {
    for (int a = 0; a < 3; ++a) p[a] = ijk[a * n + c];
  }
};

// face relation: 0 boundary, 1 same level, 2 coarser neighbour, 3 1:4 face
__device__ int relation(const View &v, int level, const int64_t w[3], int64_t *same, int64_t *coarse) {
  *same = v.find(level, w);
  if (*same >= 0) return 1;
  const int64_t wc[3] = {floordiv2(w[0]), floordiv2(w[1]), floordiv2(w[2])};
  *coarse = v.find(level - 1, wc);
  return *coarse >= 0 ? 2 : 3;
}

__global__ void k_keys(View v, uint64_t *keys, unsigned long long *err) {
  for (int64_t c = int64_t(blockIdx.x) * kBlock + threadIdx.x; c < v.n; c += int64_t(gridDim.x) * kBlock) {
    const int l = v.level[c];
    int64_t p[3];
    v.pos(c, p);
    bool ok = l >= 0 && l <= kMaxLevel;
    for (int a = 0; a < 3 && ok; ++a) ok = p[a] >= 0 && p[a] < (int64_t(1) << l);
    keys[c] = ok ? morton(l, p[0], p[1], p[2]) : 0;
    if (!ok) atomicCAS(err, 0ull, (1ull << 40) | (unsigned long long)c);
  }
}

__global__ void k_check_sorted(const uint64_t *keys, int64_t n, unsigned long long *err) {
  for (int64_t c = int64_t(blockIdx.x) * kBlock + threadIdx.x + 1; c < n; c += int64_t(gridDim.x) * kBlock)
    if (!(keys[c - 1] < keys[c])) atomicCAS(err, 0ull, (2ull << 40) | (unsigned long long)c);
}

__global__ void k_count_hang(View v, int32_t *count) {
  for (int64_t c = int64_t(blockIdx.x) * kBlock + threadIdx.x; c < v.n; c += int64_t(gridDim.x) * kBlock) {
    const int l = v.level[c];
    int64_t p[3];
    v.pos(c, p);
    int cnt = 0;
    for (int f = 0; f < 6; ++f) {
      int64_t w[3], u[3], same, coarse;
      if (!v.neighbour_pos(l, p, f, w, u)) continue;
      if (relation(v, l, w, &same, &coarse) == 3) ++cnt;
    }
    count[c] = cnt;
  }
}

// exclusive scan of count[n] in place, three passes over tiles of 1024
constexpr int kScanTile = 1024;

__global__ void k_scan_tiles(int32_t *data, int64_t n, int64_t *tile_sums) {
  __shared__ int64_t s[kScanTile];
  const int64_t base = int64_t(blockIdx.x) * kScanTile;
  const int t = threadIdx.x;
  const int64_t i = base + t;
  s[t] = i < n ? data[i] : 0;
  __syncthreads();
  for (int off = 1; off < kScanTile; off <<= 1) {  // inclusive Hillis-Steele
    const int64_t add = t >= off ? s[t - off] : 0;
    __syncthreads();
    s[t] += add;
    __syncthreads();
  }
  if (i < n) data[i] = int32_t(s[t] - (i < n ? data[i] : 0));  // exclusive within the tile
  if (t == kScanTile - 1) tile_sums[blockIdx.x] = s[t];
}

__global__ void k_scan_sums(int64_t *tile_sums, int64_t ntiles, int64_t *total) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int64_t acc = 0;
  for (int64_t b = 0; b < ntiles; ++b) {
    const int64_t v = tile_sums[b];
    tile_sums[b] = acc;
    acc += v;
  }
  *total = acc;
}

__global__ void k_scan_add(int32_t *data, int64_t n, const int64_t *tile_sums) {
  const int64_t i = int64_t(blockIdx.x) * kScanTile + threadIdx.x;
  if (i < n) data[i] += int32_t(tile_sums[blockIdx.x]);
}

__global__ void k_flatten(View v, const int32_t *offset, DevTables t, unsigned long long *err) {
  const int64_t N = v.n;
  for (int64_t c = int64_t(blockIdx.x) * kBlock + threadIdx.x; c < N; c += int64_t(gridDim.x) * kBlock) {
    const int l = v.level[c];
    int64_t pos[3];
    v.pos(c, pos);
    t.level[c] = l;
    t.vol[c] = v.volume(l, pos);
    double cc[3];
    v.centroid(l, pos, cc);
    int64_t rec = offset[c];
    for (int f = 0; f < 6; ++f) {
      const int64_t fc = int64_t(f) * N + c;
      const int a = axis_of(f);
      int64_t w[3], u[3];
      int32_t code;
      const double area = v.face_area(l, pos, f);
      double dcf = 0.0, dcc = 0.0;
      int nface = opp_of(f);
      if (!v.neighbour_pos(l, pos, f, w, u)) {
        code = -1 - v.g.side_bc[f];
        nface = -1;
      } else {
        int64_t same = -1, coarse = -1;
        const int rel = relation(v, l, w, &same, &coarse);
        double cn[3], co[3];
        if (rel == 1) {
          code = int32_t(same);
          v.centroid(l, u, cn);
          const double dx = cc[0] - cn[0], dy = cc[1] - cn[1], dz = cc[2] - cn[2];
          const double d = 0.5 * sqrt(dx * dx + dy * dy + dz * dz);
          dcf = 0.5 * d;
          dcc = d;
        } else if (rel == 2) {
          code = int32_t(coarse);
          const int64_t pp[3] = {floordiv2(pos[0]), floordiv2(pos[1]), floordiv2(pos[2])};
          const int64_t uc[3] = {floordiv2(u[0]), floordiv2(u[1]), floordiv2(u[2])};
          v.centroid(l - 1, pp, co);
          v.centroid(l - 1, uc, cn);
          const double dx = co[0] - cn[0], dy = co[1] - cn[1], dz = co[2] - cn[2];
          const double d = 0.25 * sqrt(dx * dx + dy * dy + dz * dz);
          dcf = 0.25 * d;
          dcc = 0.25 * d + 0.5 * d;
        } else {
          // the 4 children of w on the face toward this cell; child s holds
          // the corner at this cell's face node s (elconnfin.c:42-45)
          int32_t kids[4];
          bool ok = true;
          for (int s = 0; s < 4; ++s) {
            int64_t q[3];
            const int node = face_node(f, s);
            for (int x = 0; x < 3; ++x) q[x] = 2 * w[x] + ((node >> x) & 1);
            q[a] = 2 * w[a] + (sign_of(f) > 0 ? 0 : 1);
            const int64_t k = v.find(l + 1, q);
            kids[s] = int32_t(k);
            ok &= k >= 0;
          }
          if (!ok) atomicCAS(err, 0ull, (3ull << 40) | (unsigned long long)c);
          code = int32_t(-16 - rec);  // FVGPU_HANG0 - record
          for (int s = 0; s < 4; ++s) {
            // the fine neighbour's own face toward this cell, at its
            // unwrapped position (areaproperties on neigtr[f][s])
            int64_t qu[3];
            const int node = face_node(f, s);
            for (int x = 0; x < 3; ++x) qu[x] = 2 * u[x] + ((node >> x) & 1);
            qu[a] = 2 * u[a] + (sign_of(f) > 0 ? 0 : 1);
            t.hang_nbr[rec * 4 + s] = kids[s];
            t.hang_area[rec * 4 + s] = v.face_area(l + 1, qu, opp_of(f));
          }
          ++rec;
          v.centroid(l, u, cn);
          const double dx = cc[0] - cn[0], dy = cc[1] - cn[1], dz = cc[2] - cn[2];
          const double d = 0.5 * sqrt(dx * dx + dy * dy + dz * dz);
          dcf = 0.5 * d;
          dcc = 0.5 * d + 0.25 * d;
        }
      }
      t.nbr[fc] = code;
      t.nbr_face[fc] = nface;
      t.area[fc] = area;
      t.dcf[fc] = dcf;
      t.dcc[fc] = dcc;
    }
  }
}

unsigned grid_for(int64_t n) { return unsigned(n / kBlock + 1 < 152 * 16 ? n / kBlock + 1 : 152 * 16); }

}  // namespace

cudaError_t flatten_count(const LeafGeom &g, int64_t n, const int32_t *level, const int32_t *ijk, uint64_t *keys,
                          int32_t *counts, int64_t *tile_sums, int64_t *nhang, unsigned long long *err,
                          cudaStream_t st) {
  View v{g, n, level, ijk, keys};
  k_keys<<<grid_for(n), kBlock, 0, st>>>(v, keys, err);
  k_check_sorted<<<grid_for(n), kBlock, 0, st>>>(keys, n, err);
  k_count_hang<<<grid_for(n), kBlock, 0, st>>>(v, counts);
  const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
  k_scan_tiles<<<unsigned(ntiles), kScanTile, 0, st>>>(counts, n, tile_sums);
  k_scan_sums<<<1, 1, 0, st>>>(tile_sums, ntiles, nhang);
  k_scan_add<<<unsigned(ntiles), kScanTile, 0, st>>>(counts, n, tile_sums);
  return cudaGetLastError();
}

cudaError_t flatten_tables(const LeafGeom &g, int64_t n, const int32_t *level, const int32_t *ijk,
                           const uint64_t *keys, const int32_t *offsets, const DevTables &t, unsigned long long *err,
                           cudaStream_t st) {
  View v{g, n, level, ijk, keys};
  k_flatten<<<grid_for(n), kBlock, 0, st>>>(v, offsets, t, err);
  return cudaGetLastError();
}

}  // namespace fv
