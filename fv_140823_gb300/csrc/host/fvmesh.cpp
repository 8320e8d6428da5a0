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
#include "fvframes.h"

#include <algorithm>
#include <array>
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
// Element nodes of face f in face-node order, fcnd2elnd (operatetp.c:113-147,
// type 0); node n sits at offset (n & 1, n >> 1 & 1, n >> 2 & 1) in (x, y, z).
constexpr int kFaceNode[6][4] = {{0, 1, 5, 4}, {3, 7, 5, 1}, {2, 6, 7, 3},
                                 {2, 0, 4, 6}, {2, 3, 1, 0}, {6, 4, 5, 7}};

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
  // State-transfer plan of the last fvmesh_adapt: per current leaf, the leaf
  // of the mesh before it that it descends from (>= 0), or -1 - g for the
  // parent that merge group g (8 former leaves, child order) formed.
  std::vector<int32_t> src;
  std::vector<std::array<int32_t, 8>> groups;
  int64_t n_before = -1;  // leaves before the last fvmesh_adapt (-1: no plan)

  double h(int level, int a) const { return std::ldexp(len[a], -level); }
  // Coordinate of grid line I at `level` along axis a.  Because h(level+1) is
  // h(level)/2 exactly, the same physical line gets the same double at every
  // level, so parent and child corners agree bit for bit.
  double coord(int level, int a, int64_t I) const { return lo[a] + double(I) * h(level, a); }

  // Cell volume exactly as volmproperties (meshproperties.c:66-111) forms it
  // for a hexahedron: six tetrahedra on node 0, each triple product over 6.0,
  // summed in order.  On a box this can differ from hx*hy*hz in the last bit.
  double volume(int level, const int64_t p[3]) const {
    static const int kTet[6][3] = {{1, 3, 5}, {5, 3, 7}, {5, 7, 4}, {3, 2, 7}, {7, 2, 6}, {7, 6, 4}};
    double nd[8][3];
    for (int n = 0; n < 8; ++n)
      for (int a = 0; a < 3; ++a) nd[n][a] = coord(level, a, p[a] + ((n >> a) & 1));
    double vol = 0.0;
    for (int it = 0; it < 6; ++it) {
      double d[3][3];
      for (int in = 0; in < 3; ++in)
        for (int a = 0; a < 3; ++a) d[in][a] = nd[kTet[it][in]][a] - nd[0][a];
      const double c0 = d[0][1] * d[1][2] - d[0][2] * d[1][1];
      const double c1 = d[0][2] * d[1][0] - d[0][0] * d[1][2];
      const double c2 = d[0][0] * d[1][1] - d[0][1] * d[1][0];
      vol += (c0 * d[2][0] + c1 * d[2][1] + c2 * d[2][2]) / 6.0;
    }
    return vol;
  }

  // Area of face f of the cell at (level, p) exactly as areaproperties
  // (meshproperties.c:29-63) forms it from the node coordinates: the face's
  // triangles (face nodes 0,1,2 and 0,2,3), each half the norm of the cross
  // product of its edges from face node 0, summed in order.  Where the box
  // length is not a power of two the node coordinates round, and the area
  // differs from hx*hy by up to ~1e-13 relative, differently from cell to cell.
  double face_area(int level, const int64_t p[3], int f) const {
    double nd[4][3];
    for (int s = 0; s < 4; ++s)
      for (int a = 0; a < 3; ++a) nd[s][a] = coord(level, a, p[a] + ((kFaceNode[f][s] >> a) & 1));
    double area = 0.0;
    for (int it = 0; it < 2; ++it) {
      const double dx1 = nd[1 + it][0] - nd[0][0], dx2 = nd[2 + it][0] - nd[0][0];
      const double dy1 = nd[1 + it][1] - nd[0][1], dy2 = nd[2 + it][1] - nd[0][1];
      const double dz1 = nd[1 + it][2] - nd[0][2], dz2 = nd[2 + it][2] - nd[0][2];
      const double cx = dy1 * dz2 - dz1 * dy2, cy = dz1 * dx2 - dx1 * dz2, cz = dx1 * dy2 - dy1 * dx2;
      area += std::fabs(0.5 * std::sqrt(cx * cx + cy * cy + cz * cz));
    }
    return area;
  }

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

  // Face f of leaf L is a 1:4 face: its neighbour region at L's level is
  // split (neither a leaf of that level nor of the one above covers it).
  bool hanging_face(const Leaf &L, int f) const {
    int64_t w[3], u[3];
    if (!neighbour_pos(L, f, w, u)) return false;
    if (find(L.level, w) >= 0) return false;
    const int64_t q[3] = {floordiv2(w[0]), floordiv2(w[1]), floordiv2(w[2])};
    return find(L.level - 1, q) < 0;
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

  // Leaves along the Morton curve; `carry` (one entry per leaf) follows them.
  void sort_and_index(std::vector<int32_t> *carry = nullptr) {
    std::vector<std::pair<uint64_t, size_t>> tmp;
    tmp.reserve(leaves.size());
    for (size_t n = 0; n < leaves.size(); ++n) tmp.emplace_back(morton(leaves[n]), n);
    std::sort(tmp.begin(), tmp.end(),
              [](const std::pair<uint64_t, size_t> &x, const std::pair<uint64_t, size_t> &y) {
                return x.first < y.first;
              });
    std::vector<Leaf> next(leaves.size());
    for (size_t n = 0; n < tmp.size(); ++n) next[n] = leaves[tmp[n].second];
    leaves.swap(next);
    if (carry) {
      std::vector<int32_t> c(carry->size());
      for (size_t n = 0; n < tmp.size(); ++n) c[n] = (*carry)[tmp[n].second];
      carry->swap(c);
    }
    table.build(leaves);
  }

  // The 4 children of (level, p) that touch face f of a cell on the side
  // opposite to f, in sub-face order: child s holds the corner at node
  // fcnd2elnd(f, s) of that cell's face.  This is the order the reference's
  // connectivity gives the fine neighbours of a face (neigtr[f][s], kid
  // fcrefnd2elnd(ifc2, fcndrot(s, 0)) of the coarse neighbour, elconnfin.c:42-45),
  // and so the order in which their fluxes are summed.
  void near_children(int level, const int64_t p[3], int f, int64_t q[4][3]) const {
    const int a = kAxis[f];
    for (int s = 0; s < 4; ++s) {
      const int node = kFaceNode[f][s];
      for (int x = 0; x < 3; ++x) q[s][x] = 2 * p[x] + ((node >> x) & 1);
      q[s][a] = 2 * p[a] + (kSign[f] > 0 ? 0 : 1);
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

  // Splits the marked leaves into their 8 children (child ch at offset
  // bit0 = +x, bit1 = +y, bit2 = +z); children inherit the `carry` entry.
  void refine_set(const std::vector<uint8_t> &mark, std::vector<int32_t> *carry = nullptr) {
    std::vector<Leaf> next;
    std::vector<int32_t> cnext;
    const size_t grow = 7 * size_t(std::count(mark.begin(), mark.end(), 1));
    next.reserve(leaves.size() + grow);
    if (carry) cnext.reserve(leaves.size() + grow);
    for (size_t n = 0; n < leaves.size(); ++n) {
      const Leaf &L = leaves[n];
      const int nc = mark[n] ? 8 : 1;
      for (int ch = 0; ch < nc; ++ch) {
        Leaf C = L;
        if (mark[n]) {
          C.level = L.level + 1;
          for (int a = 0; a < 3; ++a) C.p[a] = 2 * L.p[a] + ((ch >> a) & 1);
        }
        next.push_back(C);
        if (carry) cnext.push_back((*carry)[n]);
      }
    }
    leaves.swap(next);
    if (carry) carry->swap(cnext);
    sort_and_index(carry);
  }

  // Refine until every face sees at most one level of difference.
  int balance(std::vector<int32_t> *carry = nullptr) {
    for (int iter = 0; iter < 64; ++iter) {
      // marking is idempotent (a leaf is marked or not, whoever marks it),
      // so the leaves are checked in parallel; marks are relaxed atomic stores
      std::vector<uint8_t> mark(leaves.size(), 0);
      bool any = false;
#pragma omp parallel for schedule(dynamic, 1024) reduction(|| : any)
      for (int64_t nn = 0; nn < int64_t(leaves.size()); ++nn) {
        const size_t n = size_t(nn);
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
              if (idx >= 0) {
                __atomic_store_n(&mark[size_t(idx)], uint8_t(1), __ATOMIC_RELAXED);
                any = true;
              }
            }
            continue;
          }
          int64_t q[4][3];
          near_children(L.level, w, f, q);
          for (int s = 0; s < 4; ++s) {
            if (find(L.level + 1, q[s]) < 0) {  // deeper than one level
              __atomic_store_n(&mark[n], uint8_t(1), __ATOMIC_RELAXED);
              any = true;
              break;
            }
          }
        }
      }
      if (!any) return 0;
      for (size_t n = 0; n < leaves.size(); ++n)
        if (mark[n] && leaves[n].level >= FVMESH_MAX_LEVEL)
          return fail(FVMESH_ERR_LEVEL, "2:1 balancing needs a level above FVMESH_MAX_LEVEL");
      refine_set(mark, carry);
    }
    return fail(FVMESH_ERR_BALANCE, "2:1 balancing did not converge");
  }

  // One adaptation pass of meshadaptation.c:23-58 from the target levels
  // `split` (criterionsplt.c), smoothed as criterionsmth.c does: a leaf
  // moves at most one level; 8 sibling leaves that all ask for a coarser
  // level merge into their parent (refineh_1.c:30-62), which keeps the
  // average of their states (merge.c:93-101); a leaf that asks for a finer
  // level splits and its children inherit its state (split.c:493); then 2:1
  // face balance.  Levels stay within [min_level, max_level].  A merge that
  // would leave the parent next to a face neighbour finer than the children
  // (now, or after this pass's splits) is skipped, so no merge is undone by
  // the balancing.
  int adapt(const int32_t *split, int min_level, int max_level) {
    const size_t n = leaves.size();
    std::vector<int8_t> dir(n, 0);  // -1 coarser, +1 finer
    for (size_t i = 0; i < n; ++i) {
      const int want = std::min(std::max(int(split[i]), min_level), max_level);
      dir[i] = want > leaves[i].level ? 1 : (want < leaves[i].level ? -1 : 0);
    }
    // merge groups: the checks read only the old leaves and dir, so each
    // leaf is tested independently; groups are then numbered in leaf order
    std::vector<int32_t> group_of(n, -1);
    std::vector<std::array<int32_t, 8>> kids_of(n);
    std::vector<uint8_t> first_child(n, 0);
    groups.clear();
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t ii = 0; ii < int64_t(n); ++ii) {
      const size_t i = size_t(ii);
      const Leaf &L = leaves[i];
      if (dir[i] >= 0 || L.level <= min_level || (L.p[0] | L.p[1] | L.p[2]) & 1) continue;
      std::array<int32_t, 8> &kids = kids_of[i];
      bool ok = true;
      for (int ch = 0; ch < 8 && ok; ++ch) {
        const int64_t q[3] = {L.p[0] + (ch & 1), L.p[1] + ((ch >> 1) & 1), L.p[2] + ((ch >> 2) & 1)};
        kids[ch] = find(L.level, q);
        ok = kids[ch] >= 0 && dir[size_t(kids[ch])] < 0;
      }
      if (!ok) continue;
      // the parent's face neighbours: no leaf finer than the children, none
      // of the children's level about to split
      Leaf P;
      P.level = L.level - 1;
      for (int a = 0; a < 3; ++a) P.p[a] = L.p[a] / 2;
      for (int f = 0; f < 6 && ok; ++f) {
        int64_t w[3], u[3];
        if (!neighbour_pos(P, f, w, u)) continue;
        if (cover_level(P.level, w) >= 0) continue;  // a leaf at the parent's level or coarser
        int64_t q[4][3];
        near_children(P.level, w, f, q);
        for (int s = 0; s < 4 && ok; ++s) {
          const int32_t k = find(L.level, q[s]);
          ok = k >= 0 && dir[size_t(k)] <= 0;
        }
      }
      if (ok) first_child[i] = 1;
    }
    for (size_t i = 0; i < n; ++i) {
      if (!first_child[i]) continue;
      for (int ch = 0; ch < 8; ++ch) group_of[size_t(kids_of[i][ch])] = int32_t(groups.size());
      groups.push_back(kids_of[i]);
    }
    std::vector<Leaf> next;
    std::vector<int32_t> carry;
    next.reserve(n);
    carry.reserve(n);
    std::vector<uint8_t> split_mark;
    for (size_t i = 0; i < n; ++i) {
      const Leaf &L = leaves[i];
      const int32_t g = group_of[i];
      if (g >= 0) {
        if (groups[size_t(g)][0] != int32_t(i)) continue;  // the first child stands for the group
        Leaf P;
        P.level = L.level - 1;
        for (int a = 0; a < 3; ++a) P.p[a] = L.p[a] / 2;
        next.push_back(P);
        carry.push_back(-1 - g);
        split_mark.push_back(0);
        continue;
      }
      next.push_back(L);
      carry.push_back(int32_t(i));
      split_mark.push_back(dir[i] > 0 && L.level < max_level ? 1 : 0);
    }
    leaves.swap(next);
    table.build(leaves);
    refine_set(split_mark, &carry);
    const int rc = balance(&carry);
    src.swap(carry);
    n_before = rc == 0 ? int64_t(n) : -1;
    return rc;
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
  const int64_t N = int64_t(m->leaves.size());
#pragma omp parallel for schedule(static) reduction(+ : nh)
  for (int64_t c = 0; c < N; ++c)
    for (int f = 0; f < 6; ++f) nh += m->hanging_face(m->leaves[size_t(c)], f) ? 1 : 0;
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

int fvmesh_leaf_cells(const fvmesh *m, int32_t *level, int32_t *ijk) {
  if (!m || !level || !ijk) return fail(FVMESH_ERR_ARG, "null argument");
  const int64_t n = int64_t(m->leaves.size());
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < n; ++c) {
    const Leaf &L = m->leaves[size_t(c)];
    level[c] = L.level;
    for (int a = 0; a < 3; ++a) ijk[a * n + c] = int32_t(L.p[a]);
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

int fvmesh_adapt(fvmesh *m, const int32_t *split, int min_level, int max_level) {
  if (!m || !split) return fail(FVMESH_ERR_ARG, "null argument");
  if (min_level < 1 || max_level > FVMESH_MAX_LEVEL || min_level > max_level)
    return fail(FVMESH_ERR_LEVEL, "need 1 <= min_level <= max_level <= FVMESH_MAX_LEVEL");
  return m->adapt(split, min_level, max_level);
}

int fvmesh_transfer(const fvmesh *m, int neq, int64_t n_old, const double *S_old, double *S_new) {
  if (!m || !S_old || !S_new || neq < 1) return fail(FVMESH_ERR_ARG, "null argument");
  if (m->n_before < 0 || n_old != m->n_before)
    return fail(FVMESH_ERR_ARG, "n_old is not the leaf count before the last fvmesh_adapt");
  const int64_t n = int64_t(m->leaves.size());
  for (int64_t i = 0; i < n; ++i) {
    const int32_t s = m->src[size_t(i)];
    for (int v = 0; v < neq; ++v) {
      const double *col = S_old + int64_t(v) * n_old;
      double x;
      if (s >= 0) {
        x = col[s];
      } else {
        // merge.c:93-101: the sum of the kids' states over nsplit, in kid order
        x = 0.0;
        for (int ch = 0; ch < 8; ++ch) x += col[m->groups[size_t(-1 - s)][size_t(ch)]] / 8.0;
      }
      S_new[int64_t(v) * n + i] = x;
    }
  }
  return 0;
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

  // Frames per face index: outward normal, t1 along the face's first edge
  // and t2, as normalvector.c / tagvector.c form them (signed zeros included)
  if (t->frames) fv_box_frames(t->frames);

  // 1:4 records are numbered in cell order: count each cell's, then number
  // them by a prefix sum, so the cells can be filled independently
  std::vector<int64_t> first(size_t(N) + 1, 0);
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < N; ++c) {
    int64_t k = 0;
    for (int f = 0; f < 6; ++f) k += m->hanging_face(m->leaves[size_t(c)], f) ? 1 : 0;
    first[size_t(c) + 1] = k;
  }
  for (int64_t c = 0; c < N; ++c) first[size_t(c) + 1] += first[size_t(c)];

  int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int64_t c = 0; c < N; ++c) {
    const Leaf &L = m->leaves[size_t(c)];
    const int l = L.level;
    const int64_t pos[3] = {L.p[0], L.p[1], L.p[2]};
    int64_t nh = first[size_t(c)];
    if (t->level) t->level[c] = l;
    if (t->ijk)
      for (int a = 0; a < 3; ++a) t->ijk[a * N + c] = L.p[a];
    if (t->vol) t->vol[c] = m->volume(l, pos);
    double cc[3];
    m->centroid(l, pos, cc);
    if (t->centroid)
      for (int a = 0; a < 3; ++a) t->centroid[a * N + c] = cc[a];

    for (int f = 0; f < 6; ++f) {
      const int64_t fc = int64_t(f) * N + c;
      int64_t w[3], u[3];
      int32_t code;
      const double area = m->face_area(l, pos, f);
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
            if (kids[s] < 0) bad = 1;  // a face sees more than one level of refinement
          }
          code = FVMESH_HANG0 - int32_t(nh);
          // areaproperties: each sub-face area is the fine neighbour's own
          // face toward this cell, at the neighbour's unwrapped position
          int64_t qu[4][3];
          m->near_children(l, u, f, qu);
          for (int s = 0; s < 4; ++s) {
            if (t->hang_nbr) t->hang_nbr[nh * 4 + s] = kids[s];
            if (t->hang_area) t->hang_area[nh * 4 + s] = m->face_area(l + 1, qu[s], kOpp[f]);
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
  if (bad) return fail(FVMESH_ERR_BALANCE, "face sees more than one level of refinement");
  return 0;
}

}  // extern "C"
