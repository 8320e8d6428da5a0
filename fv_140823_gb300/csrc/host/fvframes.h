// Face frames of the reference's hexahedron, shared by the host mesh builder
// (fvmesh.cpp) and the library's device flatten (fv_api.cu).
//
// For face f: the outward normal n, t1 along the face's first edge (face node
// 0 -> 1) and t2 from n and t1, computed the way normalvectorcalc
// (normalvector.c:46-59, with face node 2 as the third point) and
// tagvectorcalc (tagvector.c:34-56) compute them from a cell's nodes.  For
// any axis-aligned box cell the values are 0 and +-1 and do not depend on the
// cell's size or place, but the zeros carry the signs those expressions give
// (a negated zero numerator is -0.0), and the reference's own geometry holds
// exactly these bits.  Evaluated on the unit cube, node n at
// (n & 1, n >> 1 & 1, n >> 2 & 1), face nodes as fcnd2elnd
// (operatetp.c:113-147, type 0).
#pragma once

#include <math.h>

static inline void fv_box_frames(double out[54]) {
  static const int kFaceNode[6][4] = {{0, 1, 5, 4}, {3, 7, 5, 1}, {2, 6, 7, 3},
                                      {2, 0, 4, 6}, {2, 3, 1, 0}, {6, 4, 5, 7}};
  for (int f = 0; f < 6; ++f) {
    double p[3][3];
    for (int s = 0; s < 3; ++s)
      for (int a = 0; a < 3; ++a) p[s][a] = double((kFaceNode[f][s] >> a) & 1);
    const double x10 = p[1][0] - p[0][0], y10 = p[1][1] - p[0][1], z10 = p[1][2] - p[0][2];
    const double x20 = p[2][0] - p[0][0], y20 = p[2][1] - p[0][1], z20 = p[2][2] - p[0][2];
    const double cx = y10 * z20 - y20 * z10;
    const double cy = x10 * z20 - x20 * z10;
    const double cz = x10 * y20 - x20 * y10;
    const double norm = sqrt(cx * cx + cy * cy + cz * cz);
    const double nx = cx / norm, ny = -cy / norm, nz = cz / norm;
    const double norm_t = sqrt(y10 * y10 + x10 * x10 + z10 * z10);
    const double tx = x10 / norm_t, ty = y10 / norm_t, tz = z10 / norm_t;
    const double ax = ny * tz - ty * nz, ay = nx * tz - tx * nz, az = nx * ty - tx * ny;
    const double norm1 = sqrt(ax * ax + ay * ay + az * az);
    const double fr[9] = {nx, ny, nz, tx, ty, tz, ax / norm1, -ay / norm1, az / norm1};
    for (int k = 0; k < 9; ++k) out[9 * f + k] = fr[k];
  }
}
