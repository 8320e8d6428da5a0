// Host-side octree mesh builder and flattener.  See include/fvmesh.h.
//
// The reference's host keeps a forest of octrees (createtopo.c, split.c,
// elconn.c) and hands the residual a linked list of leaves whose faces point
// at 1 or 4 neighbours (`lfc_neigs`, `neigtr[f][0..3]`, `neigfc`,
// residual_faces_AMR.c:40-87).  This builder produces the same connectivity
// for an axis-aligned box: one root, uniform refinement to a base level,
// flag-driven refinement and 2:1 face balancing, leaves sorted along the
// Morton curve.  fvmesh_flatten() turns it into the SoA tables the GPU
// library consumes.
#include "fvmesh.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

thread_local std::string g_err;

int fail(int code, const char *msg) {
  g_err = msg;
  return code;
}

// Face f -> axis and outward sign; opposite face (operatetp.c:481-490).
constexpr int kAxis[6] = {1, 0, 1, 0, 2, 2};
constexpr int kSign[6] = {-1, +1, +1, -1, -1, +1};
constexpr int kOpp[6] = {2, 3, 0, 1, 5, 4};

struct Leaf {
  int32_t level;
  int32_t p[3];
};

uint64_t pack_key(int level, int64_t i, int64_t j, int64_t k) {
  return (uint64_t(level) << 57) | (uint64_t(i) << 38) | (uint64_t(j) << 19) | uint64_t(k);
}

// Open-addressing hash set of leaf keys -> leaf index.
class LeafTable {
 public:
  void build(const std::vector<Leaf> &leaves) {
    size_t cap = 16;
    while (cap < leaves.size() * 2 + 16) cap <<= 1;
    keys_.assign(cap, kEmpty);
    vals_.assign(cap, -1);
    mask_ = cap - 1;
    for (size_t n = 0; n < leaves.size(); ++n) {
      const Leaf &L = leaves[n];
      insert(pack_key(L.level, L.p[0], L.p[1], L.p[2]), int32_t(n));
    }
  }
  int32_t find(uint64_t key) const {
    size_t h = hash(key) & mask_;
    while (true) {
      uint64_t k = keys_[h];
      if (k == key) return vals_[h];
      if (k == kEmpty) return -1;
      h = (h + 1) & mask_;
    }
  }

 private:
  static constexpr uint64_t kEmpty = ~uint64_t(0);
  static uint64_t hash(uint64_t x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return x;
  }
  void insert(uint64_t key, int32_t v) {
    size_t h = hash(key) & mask_;
    while (keys_[h] != kEmpty) h = (h + 1) & mask_;
    keys_[h] = key;
    vals_[h] = v;
  }
  std::vector<uint64_t> keys_;
  std::vector<int32_t> vals_;
  size_t mask_ = 0;
};

uint64_t spread3(uint64_t x) {  // 21 bits -> every third bit
  x &= 0x1fffff;
  x = (x | x << 32) & 0x1f00000000ffffULL;
  x = (x | x << 16) & 0x1f0000ff0000ffULL;
  x = (x | x << 8) & 0x100f00f00f00f00fULL;
  x = (x | x << 4) & 0x10c30c30c30c30c3ULL;
  x = (x | x << 2) & 0x1249249249249249ULL;
  return x;
}

uint64_t morton(const Leaf &L) {
  const int sh = FVMESH_MAX_LEVEL - L.level;
  return spread3(uint64_t(L.p[0]) << sh) | (spread3(uint64_t(L.p[1]) << sh) << 1) |
         (spread3(uint64_t(L.p[2]) << sh) << 2);
}

int64_t floordiv2(int64_t a) { return a >= 0 ? a / 2 : -((-a + 1) / 2); }

}  // namespace

struct fvmesh {
  double lo[3];
  double len[3];
  int periodic[3];
  int side_bc[6];
  std::vector<Leaf> leaves;
  LeafTable table;

  double h(int level, int a) const { return std::ldexp(len[a], -level); }
  // Coordinate of grid line I at `level` along axis a.  Because h(level+1) is
  // h(level)/2 exactly, the same physical line gets the same double at every
  // level, so parent and child corners agree bit for bit.
  double coord(int level, int a, int64_t I) const { return lo[a] + double(I) * h(level, a); }

  // Cell centroid exactly as distance.c:42-56 forms it: the sum over the 8
  // local nodes of (node / 8.0), accumulated in node order.
  void centroid(int level, const int64_t p[3], double c[3]) const {
    double lohi[3][2];
    for (int a = 0; a < 3; ++a) {
      lohi[a][0] = coord(level, a, p[a]);
      lohi[a][1] = coord(level, a, p[a] + 1);
    }
    const double nd = 8.0;
    for (int a = 0; a < 3; ++a) {
      double s = 0.0;
      for (int n = 0; n < 8; ++n) s += lohi[a][(n >> a) & 1] / nd;
      c[a] = s;
    }
  }

  int32_t find(int level, const int64_t p[3]) const {
    if (level < 0) return -1;
    const int64_t n = int64_t(1) << level;
    for (int a = 0; a < 3; ++a)
      if (p[a] < 0 || p[a] >= n) return -1;
    return table.find(pack_key(level, p[0], p[1], p[2]));
  }

  // Neighbour position across face f at the cell's level.  Returns false at a
  // non-periodic domain side.  `unwrapped` keeps the image position.
  bool neighbour_pos(const Leaf &L, int f, int64_t wrapped[3], int64_t unwrapped[3]) const {
    const int a = kAxis[f];
    const int64_t n = int64_t(1) << L.level;
    for (int b = 0; b < 3; ++b) unwrapped[b] = wrapped[b] = L.p[b];
    unwrapped[a] += kSign[f];
    wrapped[a] = unwrapped[a];
    if (wrapped[a] < 0 || wrapped[a] >= n) {
      if (!periodic[a]) return false;
      wrapped[a] = (wrapped[a] + n) % n;
    }
    return true;
  }

  void sort_and_index() {
    std::vector<std::pair<uint64_t, Leaf>> tmp;
    tmp.reserve(leaves.size());
    for (const Leaf &L : leaves) tmp.emplace_back(morton(L), L);
    std::sort(tmp.begin(), tmp.end(),
              [](const std::pair<uint64_t, Leaf> &x, const std::pair<uint64_t, Leaf> &y) {
                return x.first < y.first;
              });
    for (size_t n = 0; n < tmp.size(); ++n) leaves[n] = tmp[n].second;
    table.build(leaves);
  }

  // The 4 children of (level, p) that touch face f of a cell on the `side`
  // opposite to f, in sub-face order: offsets along the two tangential axes
  // (lower axis first) 00, 10, 01, 11.
  void near_children(int level, const int64_t p[3], int f, int64_t q[4][3]) const {
    const int a = kAxis[f];
    const int b = a == 0 ? 1 : 0;
    const int c = a == 2 ? 1 : 2;
    for (int s = 0; s < 4; ++s) {
      q[s][a] = 2 * p[a] + (kSign[f] > 0 ? 0 : 1);
      q[s][b] = 2 * p[b] + (s & 1);
      q[s][c] = 2 * p[c] + (s >> 1);
    }
    (void)level;
  }

  // Leaf covering (level, p) at `level` or coarser; returns its level or -1
  // when the region is subdivided below `level`.
  int cover_level(int level, const int64_t p[3]) const {
    int64_t q[3] = {p[0], p[1], p[2]};
    for (int l = level; l >= 0; --l) {
      if (find(l, q) >= 0) return l;
      for (int a = 0; a < 3; ++a) q[a] = floordiv2(q[a]);
    }
    return -1;
  }

  void refine_set(const std::vector<uint8_t> &mark) {
    std::vector<Leaf> next;
    next.reserve(leaves.size() + 7 * size_t(std::count(mark.begin(), mark.end(), 1)));
    for (size_t n = 0; n < leaves.size(); ++n) {
      const Leaf &L = leaves[n];
      if (!mark[n]) {
        next.push_back(L);
        continue;
      }
      for (int ch = 0; ch < 8; ++ch) {
        Leaf C;
        C.level = L.level + 1;
        for (int a = 0; a < 3; ++a) C.p[a] = 2 * L.p[a] + ((ch >> a) & 1);
        next.push_back(C);
      }
    }
    leaves.swap(next);
    sort_and_index();
  }

  // Refine until every face sees at most one level of difference.
  int balance() {
    for (int iter = 0; iter < 64; ++iter) {
      std::vector<uint8_t> mark(leaves.size(), 0);
      bool any = false;
      for (size_t n = 0; n < leaves.size(); ++n) {
        const Leaf &L = leaves[n];
        for (int f = 0; f < 6; ++f) {
          int64_t w[3], u[3];
          if (!neighbour_pos(L, f, w, u)) continue;
          const int cl = cover_level(L.level, w);
          if (cl >= 0) {
            if (cl < L.level - 1) {  // the coarse neighbour must split
              int64_t q[3] = {w[0], w[1], w[2]};
              for (int l = L.level; l > cl; --l)
                for (int a = 0; a < 3; ++a) q[a] = floordiv2(q[a]);
              const int32_t idx = find(cl, q);
              if (idx >= 0 && !mark[idx]) {
                mark[idx] = 1;
                any = true;
              }
            }
            continue;
          }
          int64_t q[4][3];
          near_children(L.level, w, f, q);
          for (int s = 0; s < 4; ++s) {
            if (find(L.level + 1, q[s]) < 0) {  // deeper than one level
              if (!mark[n]) {
                mark[n] = 1;
                any = true;
              }
              break;
            }
          }
        }
      }
      if (!any) return 0;
      for (size_t n = 0; n < leaves.size(); ++n)
        if (mark[n] && leaves[n].level >= FVMESH_MAX_LEVEL)
          return fail(FVMESH_ERR_LEVEL, "2:1 balancing needs a level above FVMESH_MAX_LEVEL");
      refine_set(mark);
    }
    return fail(FVMESH_ERR_BALANCE, "2:1 balancing did not converge");
  }
};

extern "C" {

const char *fvmesh_last_error(void) { return g_err.c_str(); }

int fvmesh_create_uniform(const double lo[3], const double len[3], int base_level,
                          const int periodic[3], const int side_bc[6], fvmesh **out) {
  if (!lo || !len || !periodic || !side_bc || !out) return fail(FVMESH_ERR_ARG, "null argument");
  if (base_level < 1 || base_level > FVMESH_MAX_LEVEL)
    return fail(FVMESH_ERR_LEVEL, "base_level must lie in [1, FVMESH_MAX_LEVEL]");
  for (int a = 0; a < 3; ++a)
    if (!(len[a] > 0.0) || !std::isfinite(lo[a])) return fail(FVMESH_ERR_ARG, "bad box");
  for (int f = 0; f < 6; ++f) {
    if (periodic[kAxis[f]]) continue;
    if (side_bc[f] < 1 || side_bc[f] > 4) return fail(FVMESH_ERR_ARG, "side_bc must be 1..4");
  }
  fvmesh *m = new (std::nothrow) fvmesh();
  if (!m) return fail(FVMESH_ERR_NOMEM, "out of memory");
  for (int a = 0; a < 3; ++a) {
    m->lo[a] = lo[a];
    m->len[a] = len[a];
    m->periodic[a] = periodic[a] ? 1 : 0;
  }
  for (int f = 0; f < 6; ++f) m->side_bc[f] = m->periodic[kAxis[f]] ? 0 : side_bc[f];
  const int64_t n = int64_t(1) << base_level;
  m->leaves.resize(size_t(n * n * n));
  size_t idx = 0;
  for (int64_t k = 0; k < n; ++k)
    for (int64_t j = 0; j < n; ++j)
      for (int64_t i = 0; i < n; ++i) {
        Leaf &L = m->leaves[idx++];
        L.level = base_level;
        L.p[0] = int32_t(i);
        L.p[1] = int32_t(j);
        L.p[2] = int32_t(k);
      }
  m->sort_and_index();
  *out = m;
  return 0;
}

void fvmesh_destroy(fvmesh *m) { delete m; }

int fvmesh_domain(const fvmesh *m, double lo[3], double len[3], int periodic[3], int side_bc[6]) {
  if (!m) return fail(FVMESH_ERR_ARG, "null mesh");
  for (int a = 0; a < 3; ++a) {
    if (lo) lo[a] = m->lo[a];
    if (len) len[a] = m->len[a];
    if (periodic) periodic[a] = m->periodic[a];
  }
  if (side_bc)
    for (int f = 0; f < 6; ++f) side_bc[f] = m->side_bc[f];
  return 0;
}

int fvmesh_sizes(const fvmesh *m, int64_t *ncells, int64_t *nhang) {
  if (!m) return fail(FVMESH_ERR_ARG, "null mesh");
  int64_t nh = 0;
  for (const Leaf &L : m->leaves)
    for (int f = 0; f < 6; ++f) {
      int64_t w[3], u[3];
      if (!m->neighbour_pos(L, f, w, u)) continue;
      if (m->find(L.level, w) >= 0) continue;
      int64_t q[3] = {floordiv2(w[0]), floordiv2(w[1]), floordiv2(w[2])};
      if (m->find(L.level - 1, q) >= 0) continue;
      ++nh;
    }
  if (ncells) *ncells = int64_t(m->leaves.size());
  if (nhang) *nhang = nh;
  return 0;
}

int fvmesh_leaves(const fvmesh *m, int32_t *level, double *centroid) {
  if (!m) return fail(FVMESH_ERR_ARG, "null mesh");
  const size_t n = m->leaves.size();
  for (size_t c = 0; c < n; ++c) {
    const Leaf &L = m->leaves[c];
    if (level) level[c] = L.level;
    if (centroid) {
      int64_t p[3] = {L.p[0], L.p[1], L.p[2]};
      double x[3];
      m->centroid(L.level, p, x);
      for (int a = 0; a < 3; ++a) centroid[a * n + c] = x[a];
    }
  }
  return 0;
}

int fvmesh_refine(fvmesh *m, const uint8_t *flags, int max_level) {
  if (!m || !flags) return fail(FVMESH_ERR_ARG, "null argument");
  if (max_level > FVMESH_MAX_LEVEL) return fail(FVMESH_ERR_LEVEL, "max_level too large");
  std::vector<uint8_t> mark(m->leaves.size(), 0);
  for (size_t n = 0; n < m->leaves.size(); ++n)
    mark[n] = (flags[n] && m->leaves[n].level < max_level) ? 1 : 0;
  m->refine_set(mark);
  return m->balance();
}

int fvmesh_cell_nodes(const fvmesh *m, int level, int i, int j, int k, double xyz[8][3]) {
  if (!m || !xyz) return fail(FVMESH_ERR_ARG, "null argument");
  const int64_t p[3] = {i, j, k};
  for (int n = 0; n < 8; ++n)
    for (int a = 0; a < 3; ++a) xyz[n][a] = m->coord(level, a, p[a] + ((n >> a) & 1));
  return 0;
}

int fvmesh_flatten(const fvmesh *m, const fvmesh_tables *t) {
  if (!m || !t) return fail(FVMESH_ERR_ARG, "null argument");
  const int64_t N = int64_t(m->leaves.size());
  int64_t nh = 0;

  // Frames per face index: outward normal, t1 along the face's first edge
  // (node fcnd2elnd(f,0) -> fcnd2elnd(f,1), operatetp.c:113-147) and
  // t2 = n x t1, as normalvector.c / tagvector.c form them for a box.
  static const double kFrames[6][9] = {
      {0, -1, 0, 1, 0, 0, 0, 0, 1},   // f0 -y
      {1, 0, 0, 0, 0, 1, 0, -1, 0},   // f1 +x
      {0, 1, 0, 0, 0, 1, 1, 0, 0},    // f2 +y
      {-1, 0, 0, 0, -1, 0, 0, 0, 1},  // f3 -x
      {0, 0, -1, 1, 0, 0, 0, -1, 0},  // f4 -z
      {0, 0, 1, 0, -1, 0, 1, 0, 0},   // f5 +z
  };
  if (t->frames)
    for (int f = 0; f < 6; ++f)
      for (int q = 0; q < 9; ++q) t->frames[f * 9 + q] = kFrames[f][q] + 0.0;

  for (int64_t c = 0; c < N; ++c) {
    const Leaf &L = m->leaves[size_t(c)];
    const int l = L.level;
    const int64_t pos[3] = {L.p[0], L.p[1], L.p[2]};
    if (t->level) t->level[c] = l;
    if (t->ijk)
      for (int a = 0; a < 3; ++a) t->ijk[a * N + c] = L.p[a];
    const double hx = m->h(l, 0), hy = m->h(l, 1), hz = m->h(l, 2);
    if (t->vol) t->vol[c] = (hx * hy) * hz;
    double cc[3];
    m->centroid(l, pos, cc);
    if (t->centroid)
      for (int a = 0; a < 3; ++a) t->centroid[a * N + c] = cc[a];

    for (int f = 0; f < 6; ++f) {
      const int64_t fc = int64_t(f) * N + c;
      const int a = kAxis[f];
      const int b = a == 0 ? 1 : 0;
      const int cax = a == 2 ? 1 : 2;
      int64_t w[3], u[3];
      int32_t code;
      double area = m->h(l, b) * m->h(l, cax);
      double dcf = 0.0, dcc = 0.0;
      int nface = kOpp[f];
      if (!m->neighbour_pos(L, f, w, u)) {
        code = -1 - m->side_bc[f];
        nface = -1;
        // distance.c: the boundary neighbour is the global root (level 0),
        // so no level branch applies and both distances stay 0.
      } else {
        const int32_t same = m->find(l, w);
        int64_t wc[3] = {floordiv2(w[0]), floordiv2(w[1]), floordiv2(w[2])};
        const int32_t coarse = same >= 0 ? -1 : m->find(l - 1, wc);
        double cn[3], co[3];
        if (same >= 0) {
          code = same;
          m->centroid(l, u, cn);
          const double dx = cc[0] - cn[0], dy = cc[1] - cn[1], dz = cc[2] - cn[2];
          const double d = 0.5 * std::sqrt(dx * dx + dy * dy + dz * dz);
          dcf = 0.5 * d;
          dcc = d;
        } else if (coarse >= 0) {
          code = coarse;
          // distance.c:119-144: own parent centroid vs coarse neighbour.
          int64_t pp[3] = {floordiv2(pos[0]), floordiv2(pos[1]), floordiv2(pos[2])};
          int64_t uc[3] = {floordiv2(u[0]), floordiv2(u[1]), floordiv2(u[2])};
          m->centroid(l - 1, pp, co);
          m->centroid(l - 1, uc, cn);
          const double dx = co[0] - cn[0], dy = co[1] - cn[1], dz = co[2] - cn[2];
          const double d = 0.25 * std::sqrt(dx * dx + dy * dy + dz * dz);
          dcf = 0.25 * d;
          dcc = 0.25 * d + 0.5 * d;
        } else {
          int64_t q[4][3];
          m->near_children(l, w, f, q);
          int32_t kids[4];
          for (int s = 0; s < 4; ++s) {
            kids[s] = m->find(l + 1, q[s]);
            if (kids[s] < 0) return fail(FVMESH_ERR_BALANCE, "face sees more than one level of refinement");
          }
          code = FVMESH_HANG0 - int32_t(nh);
          const double sub = m->h(l + 1, b) * m->h(l + 1, cax);
          for (int s = 0; s < 4; ++s) {
            if (t->hang_nbr) t->hang_nbr[nh * 4 + s] = kids[s];
            if (t->hang_area) t->hang_area[nh * 4 + s] = sub;
          }
          if (t->hang_cell) t->hang_cell[nh] = int32_t(c);
          if (t->hang_face) t->hang_face[nh] = f;
          ++nh;
          // distance.c:90-116: the first fine neighbour's parent is the
          // same-level cell at the unwrapped position.
          m->centroid(l, u, cn);
          const double dx = cc[0] - cn[0], dy = cc[1] - cn[1], dz = cc[2] - cn[2];
          const double d = 0.5 * std::sqrt(dx * dx + dy * dy + dz * dz);
          dcf = 0.5 * d;
          dcc = 0.5 * d + 0.25 * d;
        }
      }
      if (t->nbr) t->nbr[fc] = code;
      if (t->nbr_face) t->nbr_face[fc] = nface;
      if (t->area) t->area[fc] = area;
      if (t->dcf) t->dcf[fc] = dcf;
      if (t->dcc) t->dcc[fc] = dcc;
    }
  }
  return 0;
}

}  // extern "C"
