// Tecplot export of a leaf field with nodes shared between leaves: the file
// the reference writes every `exstep` steps (exportfield_linked_V3.c:19-572,
// called from loop.c:50-55 after gradcalc).
//
// The file is an FEPOINT zone of BRICK elements.  Its points are "links": a
// link gathers the leaf corners that the face connectivity joins, and carries
// the mean over those corners' leaves of the conserved variables, the
// hydrostatic pressure and the magnitudes of four gradients.  To give the
// same bytes as the reference, links are formed, merged and numbered in the
// reference's order:
//   * leaves in list order, faces 0..5, face nodes 0..3 (fcnd2elnd order);
//   * across a face to a leaf of the same level, or to the fine leaf s of a
//     1:4 face at face node s, the corner is joined to the neighbour's node
//     at the same point; across a boundary or to a coarser leaf it only gets
//     a link of its own if it has none;
//   * joining two corners that both have links appends the second link's
//     members, in order, to the first; surviving links keep creation order.
// Values are accumulated as var += x / count over a link's members in that
// order, and printed with the reference's printf formats.
#include <stdio.h>

#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "fvmesh.h"

namespace {

thread_local std::string g_export_err;

int export_fail(int code, const std::string &msg) {
  g_export_err = msg;
  return code;
}

// face f -> normal axis (faces 0 = -y, 1 = +x, 2 = +y, 3 = -x, 4 = -z, 5 = +z)
constexpr int kAxis[6] = {1, 0, 1, 0, 2, 2};
// element node at face node s of face f, fcnd2elnd (operatetp.c:113-147,
// type 0); node n sits at offset (n & 1, n >> 1 & 1, n >> 2 & 1)
constexpr int kFaceNode[6][4] = {{0, 1, 5, 4}, {3, 7, 5, 1}, {2, 6, 7, 3},
                                 {2, 0, 4, 6}, {2, 3, 1, 0}, {6, 4, 5, 7}};
// Tecplot BRICK corner order in element nodes (TPNDS[.][0],
// exportfield_linked_V3.c:83-90)
constexpr int kBrickNode[8] = {0, 1, 3, 2, 4, 5, 7, 6};

uint64_t spread3(uint64_t x) {
  uint64_t r = 0;
  for (int b = 0; b < 21; ++b) r |= ((x >> b) & 1ull) << (3 * b);
  return r;
}

// Hydrostatic pressure of a leaf, volmvalues.c:3-44 (model 1), with
// barotropic_eos.c:3-30 (model 2) and barotropic_eos.c:32-129 (model 3).
// Returns false where the model-3 pressure has no real root (the reference
// prints " double nan" and exits).
bool leaf_pressure(const fvmesh_tecplot &cfg, const double *q, double &p) {
  const double r = q[0];
  if (cfg.model == 1) {
    const double u = q[1] / r, v = q[2] / r, w = q[3] / r;
    const double e_int = (q[4] / r) - 0.5 * (u * u + v * v + w * w);
    p = r * (cfg.gamma - 1.0) * e_int - cfg.gamma * cfg.pinf;
    return true;
  }
  if (cfg.model == 2) {
    const double nexp = 7.15, beta = 293526643.0, cbar = 1450.0, psat = 2339.0, rsat = 998.2;
    if (r >= rsat) p = psat + beta * (std::pow((r / rsat), nexp) - 1.0);
    if (r < rsat) p = psat + cbar * ((1.0 / rsat) - (1.0 / r));
    return true;
  }
  const double ry = q[4] / r;
  const double y = (0 > ry) ? 0 : ry;  // max(0, S[4] / r), strdata.h's macro
  const double R_G = 286.0, T_ref = 293.15, r_sat = 998.1618, p_sat = 2340.0;
  const double speeds[2] = {1482.5, 1.0};  // liquid, then the mixture fallback
  for (double c : speeds) {
    const double b = c * c * r_sat - p_sat - r * y * R_G * T_ref - r * (c * c) * (1.0 - y);
    const double d = (p_sat - c * c * r_sat) * r * y * R_G * T_ref;
    if (std::isnan(std::sqrt(b * b - 4.0 * d))) continue;
    const double p1 = (-b + std::sqrt(b * b - 4.0 * d)) / 2.0;
    const double p2 = (-b - std::sqrt(b * b - 4.0 * d)) / 2.0;
    p = (p1 > p2) ? p1 : p2;
    return true;
  }
  return false;
}

double magnitude(const double *SG, int64_t n, int row, int64_t c) {
  const double gx = SG[(int64_t(row) * 3 + 0) * n + c];
  const double gy = SG[(int64_t(row) * 3 + 1) * n + c];
  const double gz = SG[(int64_t(row) * 3 + 2) * n + c];
  return std::sqrt(gx * gx + gy * gy + gz * gz);
}

struct Corner {
  int32_t cell;
  int32_t node;
};

}  // namespace

extern "C" {

const char *fvmesh_export_last_error(void) { return g_export_err.c_str(); }

int fvmesh_export_tecplot(const fvmesh_tecplot *cfg, int64_t n, const int32_t *level, const int32_t *ijk,
                          const int32_t *nbr, const int32_t *hang_nbr, int64_t nhang, const double lo[3],
                          const double len[3], const double *S, const double *SG, const char *path) {
  if (!cfg || !level || !ijk || !nbr || !lo || !len || !S || !path || (nhang > 0 && !hang_nbr))
    return export_fail(FVMESH_ERR_ARG, "null argument");
  if (cfg->model < 1 || cfg->model > 3 || cfg->neq != (cfg->model == 2 ? 4 : 5))
    return export_fail(FVMESH_ERR_ARG, "model must be 1 (neq 5), 2 (neq 4) or 3 (neq 5)");
  // links are numbered in int32 (at most 8 per leaf), as the file's %d fields are
  if (n < 1 || n > (int64_t(1) << 27)) return export_fail(FVMESH_ERR_ARG, "leaf count out of range");
  const int neq = cfg->neq;
  const int rl = cfg->root_level;
  for (int64_t c = 0; c < n; ++c)
    if (level[c] < rl || level[c] > FVMESH_MAX_LEVEL)
      return export_fail(FVMESH_ERR_LEVEL, "a leaf is coarser than root_level");

  // -- links ---------------------------------------------------------------
  std::vector<int32_t> elnd(size_t(n) * 8, -1);
  std::vector<std::vector<Corner>> links;
  links.reserve(size_t(n) * 2);
  for (int64_t c = 0; c < n; ++c) {
    const int l = level[c];
    for (int f = 0; f < 6; ++f) {
      const int32_t code = nbr[int64_t(f) * n + c];
      const bool boundary = code < 0 && code > FVMESH_HANG0;
      const bool hanging = code <= FVMESH_HANG0;
      int64_t r = -1;
      if (hanging) {
        r = int64_t(FVMESH_HANG0) - code;
        if (r >= nhang) return export_fail(FVMESH_ERR_ARG, "hanging record out of range");
      } else if (!boundary && (code >= n)) {
        return export_fail(FVMESH_ERR_ARG, "neighbour out of range");
      }
      // joined across this face: a same-level or finer neighbour
      const bool join = hanging || (!boundary && level[code] >= l);
      for (int s = 0; s < 4; ++s) {
        const int node1 = kFaceNode[f][s];
        int32_t &link1 = elnd[size_t(c) * 8 + node1];
        if (!join) {
          if (link1 < 0) {
            link1 = int32_t(links.size());
            links.push_back({{int32_t(c), node1}});
          }
          continue;
        }
        const int32_t other = hanging ? hang_nbr[4 * r + s] : code;
        if (other < 0 || other >= n) return export_fail(FVMESH_ERR_ARG, "neighbour out of range");
        // the neighbour's node at the same point: fcrefnd2elnd(neigfc, fcndrot(s, 0))
        // for these axis-aligned leaves is the corner mirrored across the face
        const int node2 = node1 ^ (1 << kAxis[f]);
        const int32_t link2 = elnd[size_t(other) * 8 + node2];
        if (link1 < 0 && link2 < 0) {
          const int32_t id = int32_t(links.size());
          links.push_back({{int32_t(c), node1}, {other, node2}});
          link1 = id;
          elnd[size_t(other) * 8 + node2] = id;
        } else if (link1 >= 0 && link2 < 0) {
          links[size_t(link1)].push_back({other, node2});
          elnd[size_t(other) * 8 + node2] = link1;
        } else if (link1 < 0 && link2 >= 0) {
          links[size_t(link2)].push_back({int32_t(c), node1});
          link1 = link2;
        } else if (link1 != link2) {
          const int32_t keep = link1;
          std::vector<Corner> moved;
          moved.swap(links[size_t(link2)]);
          for (const Corner &k : moved) {
            elnd[size_t(k.cell) * 8 + k.node] = keep;
            links[size_t(keep)].push_back(k);
          }
        }
      }
    }
  }
  // compaction: surviving links in creation order
  std::vector<int32_t> renum(links.size(), -1);
  int64_t nlinks = 0;
  for (size_t i = 0; i < links.size(); ++i)
    if (!links[i].empty()) renum[i] = int32_t(nlinks++);
  for (int64_t k = 0; k < n * 8; ++k) {
    if (elnd[size_t(k)] < 0) return export_fail(FVMESH_ERR_ARG, "a corner has no link");
    elnd[size_t(k)] = renum[size_t(elnd[size_t(k)])];
  }

  // -- file ------------------------------------------------------------------
  FILE *fp = fopen(path, "w");
  if (!fp) return export_fail(FVMESH_ERR_ARG, std::string("cannot open ") + path);
  static const char *kVars[3] = {
      " VARIABLES =  \"X\" \"Y\" \"Z\" \"iel\" \"part\" \"rho\" \"U\" \"V\" \"W\" \"E\" \"P\" \"G_rho\" \"G_u\" "
      "\"G_v\" \"G_p\" ",
      " VARIABLES =  \"X\" \"Y\" \"Z\" \"iel\" \"part\" \"rho\" \"U\" \"V\" \"W\" \"P\" \"G_rho\" \"G_u\" \"G_v\" "
      "\"G_p\" ",
      " VARIABLES =  \"X\" \"Y\" \"Z\" \"iel\" \"part\" \"rho\" \"U\" \"V\" \"W\" \"rhoY\" \"P\" \"G_rho\" \"G_u\" "
      "\"G_v\" \"G_p\" "};
  fputs(kVars[cfg->model - 1], fp);
  fputs(" \n ", fp);
  fprintf(fp, "ZONE T=\"%d\",N=%d,E=%d,F=FEPOINT,ET=BRICK,DT=(double,double,double)\n", 1, int(nlinks), int(n));

  const int nvar = neq + 1 + 4;
  double q[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (const std::vector<Corner> &lk : links) {
    if (lk.empty()) continue;
    const double cnt = double(lk.size());
    double var[10] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (const Corner &k : lk) {
      for (int v = 0; v < neq; ++v) {
        q[v] = S[int64_t(v) * n + k.cell];
        var[v] += q[v] / cnt;
      }
      double p = 0.0;
      if (!leaf_pressure(*cfg, q, p)) {
        fclose(fp);
        return export_fail(FVMESH_ERR_ARG, "no real root of the mixture pressure at cell " + std::to_string(k.cell));
      }
      var[neq] += p / cnt;
      const double g[4] = {SG ? magnitude(SG, n, 0, k.cell) : 0.0, SG ? magnitude(SG, n, 1, k.cell) : 0.0,
                           SG ? magnitude(SG, n, 2, k.cell) : 0.0, SG ? magnitude(SG, n, neq, k.cell) : 0.0};
      for (int j = 0; j < 4; ++j) var[neq + 1 + j] += g[j] / cnt;
    }
    const Corner &k0 = lk.front();
    const int lv = level[k0.cell];
    double x[3];
    int64_t tree[3];
    for (int a = 0; a < 3; ++a) {
      const int64_t I = int64_t(ijk[int64_t(a) * n + k0.cell]) + ((k0.node >> a) & 1);
      x[a] = lo[a] + double(I) * std::ldexp(len[a], -lv);
      tree[a] = int64_t(ijk[int64_t(a) * n + k0.cell]) >> (lv - rl);
    }
    const uint64_t root = spread3(uint64_t(tree[0])) | (spread3(uint64_t(tree[1])) << 1) |
                          (spread3(uint64_t(tree[2])) << 2);
    fprintf(fp, "%e %e %e %d %d ", x[0], x[1], x[2], int(root), 0);
    for (int v = 0; v < nvar; ++v) fprintf(fp, " %e ", var[v]);
    fputs(" \n", fp);
  }
  for (int64_t c = 0; c < n; ++c) {
    for (int j = 0; j < 8; ++j) fprintf(fp, "%d ", 1 + elnd[size_t(c) * 8 + kBrickNode[j]]);
    fputs("\n", fp);
  }
  if (fclose(fp) != 0) return export_fail(FVMESH_ERR_ARG, std::string("write failed: ") + path);
  return 0;
}

}  // extern "C"
