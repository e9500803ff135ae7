// face_loads.cpp -- consistent nodal forces of face pressures (the DLOAD
// part of the right-hand side), computed on the host like the reference does
// in solve_linear -> apply_pressure (solver/src/analysis.rs:1365-1396).
//
// Face node lists follow CalculiX P1..P6 (C3D8: solver/src/elem.rs:894-901,
// C3D20: solver/src/quadratic.rs:266-273); the face winding gives the inward
// normal r_xi x r_eta, and the traction is +p n_in (positive p compresses).
// C3D8 faces use 2x2 Gauss with bilinear shapes (elem.rs:891-950), C3D20
// faces 3x3 Gauss with 8-node serendipity shapes (quadratic.rs:275-315,
// quad8_shape quadratic.rs:328-353).  Wedge faces follow extra.rs (below).
// Loads are added in list order.
#include <cmath>
#include <cstdint>

#include "../../include/axia_gpu.h"

namespace {

const int kFace8[6][4] = {{0, 1, 2, 3}, {4, 7, 6, 5}, {0, 4, 5, 1}, {1, 5, 6, 2}, {2, 6, 7, 3}, {3, 7, 4, 0}};
const int kFace20[6][8] = {{0, 1, 2, 3, 8, 9, 10, 11},   {4, 7, 6, 5, 15, 14, 13, 12},
                           {0, 4, 5, 1, 16, 12, 17, 8},  {1, 5, 6, 2, 17, 13, 18, 9},
                           {2, 6, 7, 3, 18, 14, 19, 10}, {3, 7, 4, 0, 19, 15, 16, 11}};
// corner / mid-side parametric positions of a face (4- or 8-node)
const int kFaceXi[8][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}, {0, -1}, {1, 0}, {0, 1}, {-1, 0}};

// shape values and derivatives of a 4-node (bilinear) or 8-node (serendipity) face
void face_shape(int nf, double s, double t, double* n, double (*dn)[2]) {
  for (int i = 0; i < nf; ++i) {
    const double a = kFaceXi[i][0], b = kFaceXi[i][1];
    if (nf == 4) {
      n[i] = 0.25 * (1.0 + a * s) * (1.0 + b * t);
      dn[i][0] = 0.25 * a * (1.0 + b * t);
      dn[i][1] = 0.25 * b * (1.0 + a * s);
    } else if (i < 4) {
      const double u = 1.0 + a * s, v = 1.0 + b * t;
      n[i] = 0.25 * u * v * (a * s + b * t - 1.0);
      dn[i][0] = 0.25 * a * v * (2.0 * a * s + b * t);
      dn[i][1] = 0.25 * b * u * (a * s + 2.0 * b * t);
    } else if (a == 0) {
      n[i] = 0.5 * (1.0 - s * s) * (1.0 + b * t);
      dn[i][0] = -s * (1.0 + b * t);
      dn[i][1] = 0.5 * (1.0 - s * s) * b;
    } else {
      n[i] = 0.5 * (1.0 - t * t) * (1.0 + a * s);
      dn[i][0] = 0.5 * (1.0 - t * t) * a;
      dn[i][1] = -t * (1.0 + a * s);
    }
  }
}

// Wedge faces (solver/src/extra.rs:184-195 C3D6, 869-880 C3D15): P1 and P2
// are the triangles, P3..P5 the quadrilaterals; corners first, then mid-sides.
const int kWedgeTri[2][6] = {{0, 1, 2, 6, 7, 8}, {3, 5, 4, 11, 10, 9}};
const int kWedgeQuad[3][8] = {{0, 1, 4, 3, 6, 13, 9, 12}, {1, 2, 5, 4, 7, 14, 10, 13}, {2, 0, 3, 5, 8, 12, 11, 14}};

inline void cross3(const double* u, const double* v, double* n) {
  n[0] = u[1] * v[2] - u[2] * v[1];
  n[1] = u[2] * v[0] - u[0] * v[2];
  n[2] = u[0] * v[1] - u[1] * v[0];
}

// One wedge face into fe (element-local, 3 per node).  The traction is
// -p r_xi x r_eta, the wedge lists winding outward (extra.rs:197-253 and
// 882-954): flat triangle = a third of -p * area vector per corner; 6-node
// triangle = 3 points of weight 1/6; quadrilaterals = 2x2 / 3x3 Gauss.
void wedge_face(int nn, int fid, const double* coords, const int32_t* c, double p, double* fe) {
  const bool quad = fid >= 3;
  const int* fl = quad ? kWedgeQuad[fid - 3] : kWedgeTri[fid - 1];
  const int nf = quad ? (nn == 6 ? 4 : 8) : (nn == 6 ? 3 : 6);
  double x[8][3];
  for (int a = 0; a < nf; ++a)
    for (int q = 0; q < 3; ++q) x[a][q] = coords[3 * (int64_t)c[fl[a]] + q];
  if (nf == 3) {
    const double u[3] = {x[1][0] - x[0][0], x[1][1] - x[0][1], x[1][2] - x[0][2]};
    const double v[3] = {x[2][0] - x[0][0], x[2][1] - x[0][1], x[2][2] - x[0][2]};
    double nrm[3];
    cross3(u, v, nrm);
    const double sc = -p * 0.5 / 3.0;
    for (int a = 0; a < 3; ++a)
      for (int q = 0; q < 3; ++q) fe[3 * fl[a] + q] += sc * nrm[q];
    return;
  }
  if (nf == 6) {
    const double pts[3][2] = {{1.0 / 6.0, 1.0 / 6.0}, {2.0 / 3.0, 1.0 / 6.0}, {1.0 / 6.0, 2.0 / 3.0}};
    for (const auto& g : pts) {
      const double l1 = g[0], l2 = g[1], l3 = 1.0 - l1 - l2;
      const double n[6] = {l1 * (2.0 * l1 - 1.0), l2 * (2.0 * l2 - 1.0), l3 * (2.0 * l3 - 1.0),
                           4.0 * l1 * l2,         4.0 * l2 * l3,         4.0 * l3 * l1};
      const double d1[6] = {4.0 * l1 - 1.0, 0.0, -(4.0 * l3 - 1.0), 4.0 * l2, -4.0 * l2, 4.0 * (l3 - l1)};
      const double d2[6] = {0.0, 4.0 * l2 - 1.0, -(4.0 * l3 - 1.0), 4.0 * l1, 4.0 * (l3 - l2), -4.0 * l1};
      double rs[3] = {0, 0, 0}, rt[3] = {0, 0, 0}, nrm[3];
      for (int a = 0; a < 6; ++a)
        for (int q = 0; q < 3; ++q) {
          rs[q] += d1[a] * x[a][q];
          rt[q] += d2[a] * x[a][q];
        }
      cross3(rs, rt, nrm);
      for (int a = 0; a < 6; ++a)
        for (int q = 0; q < 3; ++q) fe[3 * fl[a] + q] += -p * n[a] * nrm[q] * (1.0 / 6.0);
    }
    return;
  }
  const double g2 = 0.5773502691896257;
  const double g3[3] = {-0.7745966692414834, 0.0, 0.7745966692414834};
  const double w3[3] = {0.5555555555555556, 0.8888888888888888, 0.5555555555555556};
  const int m = nf == 4 ? 2 : 3;
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j) {
      const double s = nf == 4 ? (i ? g2 : -g2) : g3[i], t = nf == 4 ? (j ? g2 : -g2) : g3[j];
      double n[8], dn[8][2], rs[3] = {0, 0, 0}, rt[3] = {0, 0, 0}, nrm[3];
      face_shape(nf, s, t, n, dn);
      for (int a = 0; a < nf; ++a)
        for (int q = 0; q < 3; ++q) {
          rs[q] += dn[a][0] * x[a][q];
          rt[q] += dn[a][1] * x[a][q];
        }
      cross3(rs, rt, nrm);
      if (nf == 4) {
        for (int a = 0; a < 4; ++a)
          for (int q = 0; q < 3; ++q) fe[3 * fl[a] + q] += -p * n[a] * nrm[q];
      } else {
        const double w = w3[i] * w3[j];
        for (int a = 0; a < 8; ++a)
          for (int q = 0; q < 3; ++q) fe[3 * fl[a] + q] += -p * n[a] * nrm[q] * w;
      }
    }
}

}  // namespace

extern "C" int32_t axia_face_loads(int32_t nn, int64_t n_nodes, const double* coords, const int32_t* conn,
                                   int64_t n_loads, const int64_t* elem, const int32_t* face, const double* p,
                                   double* f_full, int64_t* bad_load) {
  if (bad_load) *bad_load = -1;
  if ((nn != 4 && nn != 6 && nn != 8 && nn != 10 && nn != 15 && nn != 20) || n_loads < 0 ||
      (n_loads > 0 && (!coords || !conn || !elem || !face || !p || !f_full)))
    return AXIA_ERR_INVALID_ARG;
  // apply_pressure has no tetrahedron arm (analysis.rs:1447): a face pressure on
  // C3D4 / C3D10 adds nothing, as in the reference
  if (nn == 4 || nn == 10) return AXIA_OK;
  if (nn == 6 || nn == 15) {
    for (int64_t k = 0; k < n_loads; ++k) {
      const int fid = face[k];
      if (fid < 1 || fid > 5 || !std::isfinite(p[k])) {
        if (bad_load) *bad_load = k;
        return fid < 1 || fid > 5 ? AXIA_ERR_INVALID_ARG : AXIA_ERR_NONFINITE;
      }
      const int32_t* c = conn + elem[k] * nn;
      for (int a = 0; a < nn; ++a)
        if (c[a] < 0 || c[a] >= n_nodes) {
          if (bad_load) *bad_load = k;
          return AXIA_ERR_INVALID_ARG;
        }
      double fe[45] = {};
      wedge_face(nn, fid, coords, c, p[k], fe);
      for (int a = 0; a < nn; ++a)
        for (int q = 0; q < 3; ++q) f_full[3 * (int64_t)c[a] + q] += fe[3 * a + q];
    }
    return AXIA_OK;
  }
  const int nf = nn == 8 ? 4 : 8;
  const double g2 = 0.5773502691896257;
  const double g3[3] = {-0.7745966692414834, 0.0, 0.7745966692414834};
  const double w3[3] = {0.5555555555555556, 0.8888888888888888, 0.5555555555555556};
  double gs[9], gt[9], gw[9];
  int ng = 0;
  if (nf == 4) {
    const double q[2] = {-g2, g2};
    for (double s : q)
      for (double t : q) gs[ng] = s, gt[ng] = t, gw[ng++] = 1.0;
  } else {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) gs[ng] = g3[i], gt[ng] = g3[j], gw[ng++] = w3[i] * w3[j];
  }
  for (int64_t k = 0; k < n_loads; ++k) {
    const int fid = face[k];
    if (fid < 1 || fid > 6 || !std::isfinite(p[k])) {
      if (bad_load) *bad_load = k;
      return fid < 1 || fid > 6 ? AXIA_ERR_INVALID_ARG : AXIA_ERR_NONFINITE;
    }
    const int32_t* c = conn + elem[k] * nn;
    const int* fl = nn == 8 ? kFace8[fid - 1] : kFace20[fid - 1];
    double x[8][3];
    for (int a = 0; a < nf; ++a) {
      const int64_t node = c[fl[a]];
      if (node < 0 || node >= n_nodes) {
        if (bad_load) *bad_load = k;
        return AXIA_ERR_INVALID_ARG;
      }
      for (int q = 0; q < 3; ++q) x[a][q] = coords[3 * node + q];
    }
    double fe[8][3] = {};
    for (int g = 0; g < ng; ++g) {
      double n[8], dn[8][2];
      face_shape(nf, gs[g], gt[g], n, dn);
      double rs[3] = {0, 0, 0}, rt[3] = {0, 0, 0};
      for (int a = 0; a < nf; ++a)
        for (int q = 0; q < 3; ++q) {
          rs[q] += dn[a][0] * x[a][q];
          rt[q] += dn[a][1] * x[a][q];
        }
      const double nrm[3] = {rs[1] * rt[2] - rs[2] * rt[1], rs[2] * rt[0] - rs[0] * rt[2],
                             rs[0] * rt[1] - rs[1] * rt[0]};
      const double sc = p[k] * gw[g];
      for (int a = 0; a < nf; ++a)
        for (int q = 0; q < 3; ++q) fe[a][q] += n[a] * (sc * nrm[q]);
    }
    for (int a = 0; a < nf; ++a)
      for (int q = 0; q < 3; ++q) f_full[3 * (int64_t)c[fl[a]] + q] += fe[a][q];
  }
  return AXIA_OK;
}
