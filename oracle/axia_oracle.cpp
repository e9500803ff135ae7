// axia_oracle.cpp -- CPU restatement of the Axia linear-static path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle: the parity tests, the
// smoke check and the CPU-baseline leg of bench.py call it as the checker.
// The product library (libaxia_gpu.so) never links, loads or calls it.
//
// It restates, in plain C++17 / FP64 and in the reference's loop order, the
// Rust functions of larsmei/axia-fem (crate axia-fem 1.31.10) on the *STATIC
// path for C3D8 / C3D20:
//   solver/src/elem.rs        invert3 (10-29), d_iso_3d (41-59),
//                             gemm_bt_d_b (90-112), fill_b3 (114-132),
//                             HEX_XI / hex8_shape / hex8_dndx (147-192),
//                             hex8_stiffness(_d) (194-219),
//                             hex8_face_pressure (891-950)
//   solver/src/quadratic.rs   G3/W3 (10-11), HEX20_XI (13-34),
//                             hex20_shape / hex20_dndx (36-98),
//                             hex_gauss (100-120), hex20_stiffness (122-146),
//                             HEX20_FACE / hex20_face_pressure (265-315),
//                             quad8_shape (328-353)
//   solver/src/analysis.rs    prescribed "last BC wins" (556-565),
//                             pin_unused_dofs isolated nodes (2283-2330),
//                             element loop + triplet push (574-668),
//                             autospc_null_diag (2164-2228),
//                             reduce / solve_kff / reconstruct (1018-1025)
//   solver/src/constraint.rs  DofMap::build (26-136, prescribed subset),
//                             DofMap::reduce (138-172), reconstruct (207-217)
//   solver/src/linalg.rs      csr_from_triplets (10-38), matvec (41-50),
//                             diag (52-63), chol_solve (78-117), pcg (199-259),
//                             residual_of (268-278)
//   solver/src/sparse_native.rs residual_ok (1572-1578)
//   solver/src/elem.rs        tet4_stiffness (221-248), tet4_nodal_stress (781-795)
//   solver/src/extra.rs       invert_n (8-49), hex8i_stiffness (256-388), hex8i_nodal_stress
//                             (390-395, = hex8_nodal_stress), hex8r_stiffness (400-457),
//                             hex8r_nodal_stress (460-472), wedge_shape / wedge6_stiffness /
//                             wedge6_nodal_stress / wedge6_face_pressure (64-255),
//                             wedge15_* (701-955)
//   solver/src/quadratic.rs   tet10_shape / tet10_dndx / tet10_stiffness (546-627),
//                             tet10_nodal_stress (678-702)
// The compliance-gradient routine at the end has no reference counterpart:
// the reference has no adjoint code.  It restates dC/drho_e =
// -p rho_e^(p-1) E0 u_e^T K_e(E=1) u_e on top of the restated hex8 stiffness.
//
// Build: oracle/build_oracle.sh (g++ -O2 -ffp-contract=off, so that products
// and sums round separately, as rustc emits them).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

enum Status : int {
  OK = 0,
  ERR_INVALID_ARG = 1,
  ERR_SINGULAR_JACOBIAN = 2,
  ERR_NEG_JACOBIAN = 3,
  ERR_MATERIAL = 4,
  ERR_NOT_CONVERGED = 5,
  ERR_ZERO_PIVOT = 6,
  ERR_INDEFINITE = 7,
  ERR_SINGULAR = 8,
  ERR_NO_FREE_DOF = 9,
};

const double G2 = 0.5773502691896257;  // elem.rs:8
const double G3[3] = {-0.7745966692414834, 0.0, 0.7745966692414834};  // quadratic.rs:10
const double W3[3] = {0.5555555555555556, 0.8888888888888888, 0.5555555555555556};  // quadratic.rs:11

const double HEX_XI[8][3] = {  // elem.rs:147-156
    {-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
    {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};

const double HEX20_XI[20][3] = {  // quadratic.rs:13-34
    {-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1}, {-1, -1, 1},
    {1, -1, 1},   {1, 1, 1},   {-1, 1, 1}, {0, -1, -1}, {1, 0, -1},
    {0, 1, -1},   {-1, 0, -1}, {0, -1, 1}, {1, 0, 1},   {0, 1, 1},
    {-1, 0, 1},   {-1, -1, 0}, {1, -1, 0}, {1, 1, 0},   {-1, 1, 0}};

const int HEX8_FACE[6][4] = {  // elem.rs:894-901
    {0, 1, 2, 3}, {4, 7, 6, 5}, {0, 4, 5, 1}, {1, 5, 6, 2}, {2, 6, 7, 3}, {3, 7, 4, 0}};

const int HEX20_FACE[6][8] = {  // quadratic.rs:266-273
    {0, 1, 2, 3, 8, 9, 10, 11},     {4, 7, 6, 5, 15, 14, 13, 12},
    {0, 4, 5, 1, 16, 12, 17, 8},    {1, 5, 6, 2, 17, 13, 18, 9},
    {2, 6, 7, 3, 18, 14, 19, 10},   {3, 7, 4, 0, 19, 15, 16, 11}};

const double QUAD_XI[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};  // elem.rs:250
const double QUAD8_XI[8][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1},
                               {0, -1},  {1, 0},  {0, 1}, {-1, 0}};  // quadratic.rs:316-325

// elem.rs:10-29
int invert3(const double a[3][3], double b[3][3], double* det_out) {
  double det = a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) -
               a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
               a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
  if (std::fabs(det) < 1e-18) return ERR_SINGULAR_JACOBIAN;
  double inv_det = 1.0 / det;
  b[0][0] = (a[1][1] * a[2][2] - a[1][2] * a[2][1]) * inv_det;
  b[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) * inv_det;
  b[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) * inv_det;
  b[1][0] = (a[1][2] * a[2][0] - a[1][0] * a[2][2]) * inv_det;
  b[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) * inv_det;
  b[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) * inv_det;
  b[2][0] = (a[1][0] * a[2][1] - a[1][1] * a[2][0]) * inv_det;
  b[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) * inv_det;
  b[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) * inv_det;
  *det_out = det;
  return OK;
}

// elem.rs:41-59
int d_iso_3d(double e, double nu, double d[36]) {
  if (nu >= 0.5 || nu <= -1.0) return ERR_MATERIAL;
  if (e <= 0.0) return ERR_MATERIAL;
  double lam = e * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
  double mu = e / (2.0 * (1.0 + nu));
  for (int i = 0; i < 36; ++i) d[i] = 0.0;
  double diag = lam + 2.0 * mu;
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) d[i * 6 + j] = (i == j) ? diag : lam;
    d[(i + 3) * 6 + (i + 3)] = mu;
  }
  return OK;
}

// elem.rs:90-112 -- tmp = D*B, ke += w * B^T * tmp (dense, as written)
void gemm_bt_d_b(double* ke, int n, const double* b, int nrow, const double* d, double w,
                 std::vector<double>& tmp) {
  tmp.assign((size_t)nrow * n, 0.0);
  for (int i = 0; i < nrow; ++i)
    for (int j = 0; j < n; ++j) {
      double s = 0.0;
      for (int k = 0; k < nrow; ++k) s += d[i * nrow + k] * b[k * n + j];
      tmp[(size_t)i * n + j] = s;
    }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double s = 0.0;
      for (int k = 0; k < nrow; ++k) s += b[k * n + i] * tmp[(size_t)k * n + j];
      ke[(size_t)i * n + j] += w * s;
    }
}

// elem.rs:114-132
void fill_b3(double* b, int nnode, const double (*dndx)[3]) {
  int n = 3 * nnode;
  for (int i = 0; i < nnode; ++i) {
    int c = 3 * i;
    double dx = dndx[i][0], dy = dndx[i][1], dz = dndx[i][2];
    b[0 * n + c] = dx;
    b[1 * n + c + 1] = dy;
    b[2 * n + c + 2] = dz;
    b[3 * n + c] = dy;
    b[3 * n + c + 1] = dx;
    b[4 * n + c + 1] = dz;
    b[4 * n + c + 2] = dy;
    b[5 * n + c] = dz;
    b[5 * n + c + 2] = dx;
  }
}

// elem.rs:158-171
void hex8_shape(double xi, double eta, double zeta, double n[8], double dn[8][3]) {
  for (int i = 0; i < 8; ++i) {
    double x = HEX_XI[i][0], e = HEX_XI[i][1], z = HEX_XI[i][2];
    n[i] = 0.125 * (1.0 + x * xi) * (1.0 + e * eta) * (1.0 + z * zeta);
    dn[i][0] = 0.125 * x * (1.0 + e * eta) * (1.0 + z * zeta);
    dn[i][1] = 0.125 * e * (1.0 + x * xi) * (1.0 + z * zeta);
    dn[i][2] = 0.125 * z * (1.0 + x * xi) * (1.0 + e * eta);
  }
}

// quadratic.rs:36-73
void hex20_shape(double xi, double eta, double zeta, double n[20], double dn[20][3]) {
  for (int i = 0; i < 8; ++i) {
    double x = HEX20_XI[i][0], e = HEX20_XI[i][1], z = HEX20_XI[i][2];
    double a = 1.0 + x * xi, b = 1.0 + e * eta, c = 1.0 + z * zeta;
    n[i] = 0.125 * a * b * c * (x * xi + e * eta + z * zeta - 2.0);
    dn[i][0] = 0.125 * x * b * c * (2.0 * x * xi + e * eta + z * zeta - 1.0);
    dn[i][1] = 0.125 * e * a * c * (x * xi + 2.0 * e * eta + z * zeta - 1.0);
    dn[i][2] = 0.125 * z * a * b * (x * xi + e * eta + 2.0 * z * zeta - 1.0);
  }
  for (int i = 8; i < 20; ++i) {
    double x = HEX20_XI[i][0], e = HEX20_XI[i][1], z = HEX20_XI[i][2];
    if (std::fabs(x) < 0.5) {
      n[i] = 0.25 * (1.0 - xi * xi) * (1.0 + e * eta) * (1.0 + z * zeta);
      dn[i][0] = 0.25 * (-2.0 * xi) * (1.0 + e * eta) * (1.0 + z * zeta);
      dn[i][1] = 0.25 * (1.0 - xi * xi) * e * (1.0 + z * zeta);
      dn[i][2] = 0.25 * (1.0 - xi * xi) * (1.0 + e * eta) * z;
    } else if (std::fabs(e) < 0.5) {
      n[i] = 0.25 * (1.0 - eta * eta) * (1.0 + x * xi) * (1.0 + z * zeta);
      dn[i][0] = 0.25 * (1.0 - eta * eta) * x * (1.0 + z * zeta);
      dn[i][1] = 0.25 * (-2.0 * eta) * (1.0 + x * xi) * (1.0 + z * zeta);
      dn[i][2] = 0.25 * (1.0 - eta * eta) * (1.0 + x * xi) * z;
    } else {
      n[i] = 0.25 * (1.0 - zeta * zeta) * (1.0 + x * xi) * (1.0 + e * eta);
      dn[i][0] = 0.25 * (1.0 - zeta * zeta) * x * (1.0 + e * eta);
      dn[i][1] = 0.25 * (1.0 - zeta * zeta) * (1.0 + x * xi) * e;
      dn[i][2] = 0.25 * (-2.0 * zeta) * (1.0 + x * xi) * (1.0 + e * eta);
    }
  }
}

// elem.rs:173-192 / quadratic.rs:75-98: J[q][p] = sum_a dN_a/dxi_p x_a,q;
// dN/dx = J^-T dN/dxi.
template <int NN>
int hex_dndx(const double* xyz, const double dn[NN][3], double dndx[NN][3], double* det) {
  double j[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int a = 0; a < NN; ++a)
    for (int p = 0; p < 3; ++p)
      for (int q = 0; q < 3; ++q) j[q][p] += dn[a][p] * xyz[3 * a + q];
  double inv[3][3];
  int st = invert3(j, inv, det);
  if (st) return st;
  for (int a = 0; a < NN; ++a)
    for (int i = 0; i < 3; ++i)
      dndx[a][i] = inv[0][i] * dn[a][0] + inv[1][i] * dn[a][1] + inv[2][i] * dn[a][2];
  return OK;
}

// elem.rs:199-219
int hex8_stiffness_d(const double* xyz, const double d[36], double* ke, double* vol_out) {
  const int n = 24;
  std::fill(ke, ke + n * n, 0.0);
  double vol = 0.0;
  const double pts[2] = {-G2, G2};
  std::vector<double> b(6 * n), tmp;
  for (double xi : pts)
    for (double eta : pts)
      for (double zeta : pts) {
        double N[8], dn[8][3], dndx[8][3], det;
        hex8_shape(xi, eta, zeta, N, dn);
        int st = hex_dndx<8>(xyz, dn, dndx, &det);
        if (st) return st;
        if (det <= 0.0) return ERR_NEG_JACOBIAN;
        std::fill(b.begin(), b.end(), 0.0);
        fill_b3(b.data(), 8, dndx);
        gemm_bt_d_b(ke, n, b.data(), 6, d, det, tmp);
        vol += det;
      }
  *vol_out = vol;
  return OK;
}

// quadratic.rs:100-120
void hex_gauss(bool reduced, std::vector<double>& pts /* xi,eta,zeta,w */) {
  pts.clear();
  if (reduced) {
    const double g[2] = {-G2, G2};
    for (double xi : g)
      for (double eta : g)
        for (double zeta : g) pts.insert(pts.end(), {xi, eta, zeta, 1.0});
  } else {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) pts.insert(pts.end(), {G3[i], G3[j], G3[k], W3[i] * W3[j] * W3[k]});
  }
}

// quadratic.rs:122-146
int hex20_stiffness(const double* xyz, double e, double nu, bool reduced, double* ke, double* vol_out) {
  double d[36];
  int st = d_iso_3d(e, nu, d);
  if (st) return st;
  const int n = 60;
  std::fill(ke, ke + n * n, 0.0);
  double vol = 0.0;
  std::vector<double> gp, b(6 * n), tmp;
  hex_gauss(reduced, gp);
  for (size_t g = 0; g < gp.size(); g += 4) {
    double N[20], dn[20][3], dndx[20][3], det;
    hex20_shape(gp[g], gp[g + 1], gp[g + 2], N, dn);
    st = hex_dndx<20>(xyz, dn, dndx, &det);
    if (st) return st;
    if (det <= 0.0) return ERR_NEG_JACOBIAN;
    std::fill(b.begin(), b.end(), 0.0);
    fill_b3(b.data(), 20, dndx);
    gemm_bt_d_b(ke, n, b.data(), 6, d, gp[g + 3] * det, tmp);
    vol += gp[g + 3] * det;
  }
  *vol_out = vol;
  return OK;
}

// elem.rs:891-950
int hex8_face_pressure(const double* xyz, int face, double p, double fe[24]) {
  if (face < 1 || face > 6) return ERR_INVALID_ARG;
  int fi = face - 1;
  for (int i = 0; i < 24; ++i) fe[i] = 0.0;
  const double pts[2] = {-G2, G2};
  for (double xi : pts)
    for (double eta : pts) {
      double n[4], dnxi[4], dneta[4];
      for (int i = 0; i < 4; ++i) {
        double x = QUAD_XI[i][0], e = QUAD_XI[i][1];
        n[i] = 0.25 * (1.0 + x * xi) * (1.0 + e * eta);
        dnxi[i] = 0.25 * x * (1.0 + e * eta);
        dneta[i] = 0.25 * e * (1.0 + x * xi);
      }
      double rxi[3] = {0, 0, 0}, reta[3] = {0, 0, 0};
      for (int a = 0; a < 4; ++a) {
        const double* q = xyz + 3 * HEX8_FACE[fi][a];
        for (int k = 0; k < 3; ++k) {
          rxi[k] += dnxi[a] * q[k];
          reta[k] += dneta[a] * q[k];
        }
      }
      double nx = rxi[1] * reta[2] - rxi[2] * reta[1];
      double ny = rxi[2] * reta[0] - rxi[0] * reta[2];
      double nz = rxi[0] * reta[1] - rxi[1] * reta[0];
      double tx = p * nx, ty = p * ny, tz = p * nz;
      for (int a = 0; a < 4; ++a) {
        int gd = 3 * HEX8_FACE[fi][a];
        fe[gd] += n[a] * tx;
        fe[gd + 1] += n[a] * ty;
        fe[gd + 2] += n[a] * tz;
      }
    }
  return OK;
}

// quadratic.rs:328-353
void quad8_shape(double xi, double eta, double n[8], double dn[8][2]) {
  for (int i = 0; i < 4; ++i) {
    double x = QUAD8_XI[i][0], e = QUAD8_XI[i][1];
    double a = 1.0 + x * xi, b = 1.0 + e * eta;
    n[i] = 0.25 * a * b * (x * xi + e * eta - 1.0);
    dn[i][0] = 0.25 * x * b * (2.0 * x * xi + e * eta);
    dn[i][1] = 0.25 * e * a * (x * xi + 2.0 * e * eta);
  }
  for (int i = 4; i < 8; ++i) {
    double x = QUAD8_XI[i][0], e = QUAD8_XI[i][1];
    if (std::fabs(x) < 0.5) {
      n[i] = 0.5 * (1.0 - xi * xi) * (1.0 + e * eta);
      dn[i][0] = -xi * (1.0 + e * eta);
      dn[i][1] = 0.5 * (1.0 - xi * xi) * e;
    } else {
      n[i] = 0.5 * (1.0 - eta * eta) * (1.0 + x * xi);
      dn[i][0] = 0.5 * (1.0 - eta * eta) * x;
      dn[i][1] = -eta * (1.0 + x * xi);
    }
  }
}

// quadratic.rs:275-315
int hex20_face_pressure(const double* xyz, int face, double p, double fe[60]) {
  if (face < 1 || face > 6) return ERR_INVALID_ARG;
  int fi = face - 1;
  for (int i = 0; i < 60; ++i) fe[i] = 0.0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double xi = G3[i], eta = G3[j], w = W3[i] * W3[j];
      double nshp[8], dn[8][2];
      quad8_shape(xi, eta, nshp, dn);
      double rxi[3] = {0, 0, 0}, reta[3] = {0, 0, 0};
      for (int a = 0; a < 8; ++a) {
        const double* q = xyz + 3 * HEX20_FACE[fi][a];
        for (int k = 0; k < 3; ++k) {
          rxi[k] += dn[a][0] * q[k];
          reta[k] += dn[a][1] * q[k];
        }
      }
      double nx = rxi[1] * reta[2] - rxi[2] * reta[1];
      double ny = rxi[2] * reta[0] - rxi[0] * reta[2];
      double nz = rxi[0] * reta[1] - rxi[1] * reta[0];
      double tx = p * nx * w, ty = p * ny * w, tz = p * nz * w;
      for (int a = 0; a < 8; ++a) {
        int gd = 3 * HEX20_FACE[fi][a];
        fe[gd] += nshp[a] * tx;
        fe[gd + 1] += nshp[a] * ty;
        fe[gd + 2] += nshp[a] * tz;
      }
    }
  return OK;
}

// elem.rs:221-248: constant-strain tetrahedron, J from the edge vectors,
// Ke = vol B^T D B with vol = det / 6
int tet4_dndx(const double* xyz, double dndx[4][3], double* det_out) {
  double j[3][3];
  for (int p = 0; p < 3; ++p)
    for (int q = 0; q < 3; ++q) j[q][p] = xyz[3 * (p + 1) + q] - xyz[q];
  double inv[3][3], det;
  int st = invert3(j, inv, &det);
  if (st) return st;
  if (det <= 0.0) return ERR_NEG_JACOBIAN;
  const double dn[4][3] = {{-1.0, -1.0, -1.0}, {1.0, 0.0, 0.0}, {0.0, 1.0, 0.0}, {0.0, 0.0, 1.0}};
  for (int a = 0; a < 4; ++a)
    for (int i = 0; i < 3; ++i) dndx[a][i] = inv[0][i] * dn[a][0] + inv[1][i] * dn[a][1] + inv[2][i] * dn[a][2];
  *det_out = det;
  return OK;
}

int tet4_stiffness(const double* xyz, double e, double nu, double* ke, double* vol_out) {
  double dndx[4][3], det;
  int st = tet4_dndx(xyz, dndx, &det);
  if (st) return st;
  const double vol = det / 6.0;
  double d[36];
  st = d_iso_3d(e, nu, d);
  if (st) return st;
  const int n = 12;
  std::fill(ke, ke + n * n, 0.0);
  std::vector<double> b(6 * n, 0.0), tmp;
  fill_b3(b.data(), 4, dndx);
  gemm_bt_d_b(ke, n, b.data(), 6, d, vol, tmp);
  *vol_out = vol;
  return OK;
}

// quadratic.rs:546-580: quadratic tetrahedron in volume coordinates
void tet10_shape(double r, double s, double t, double n[10], double dn[10][3]) {
  const double l1 = 1.0 - r - s - t, l2 = r, l3 = s, l4 = t;
  n[0] = l1 * (2.0 * l1 - 1.0);
  n[1] = l2 * (2.0 * l2 - 1.0);
  n[2] = l3 * (2.0 * l3 - 1.0);
  n[3] = l4 * (2.0 * l4 - 1.0);
  n[4] = 4.0 * l1 * l2;
  n[5] = 4.0 * l2 * l3;
  n[6] = 4.0 * l3 * l1;
  n[7] = 4.0 * l1 * l4;
  n[8] = 4.0 * l2 * l4;
  n[9] = 4.0 * l3 * l4;
  const double d1 = 4.0 * l1 - 1.0, d2 = 4.0 * l2 - 1.0, d3 = 4.0 * l3 - 1.0, d4 = 4.0 * l4 - 1.0;
  const double t_[10][3] = {{-d1, -d1, -d1},
                            {d2, 0.0, 0.0},
                            {0.0, d3, 0.0},
                            {0.0, 0.0, d4},
                            {4.0 * (l1 - l2), -4.0 * l2, -4.0 * l2},
                            {4.0 * l3, 4.0 * l2, 0.0},
                            {-4.0 * l3, 4.0 * (l1 - l3), -4.0 * l3},
                            {-4.0 * l4, -4.0 * l4, 4.0 * (l1 - l4)},
                            {4.0 * l4, 0.0, 4.0 * l2},
                            {0.0, 4.0 * l4, 4.0 * l3}};
  for (int a = 0; a < 10; ++a)
    for (int p = 0; p < 3; ++p) dn[a][p] = t_[a][p];
}

const double TET_A = 0.5854101966249685, TET_B = 0.1381966011250105;  // quadratic.rs:611-612
const double TET_PTS[4][3] = {{TET_B, TET_B, TET_B}, {TET_A, TET_B, TET_B}, {TET_B, TET_A, TET_B}, {TET_B, TET_B, TET_A}};

// quadratic.rs:607-627
int tet10_stiffness(const double* xyz, double e, double nu, double* ke, double* vol_out) {
  double d[36];
  int st = d_iso_3d(e, nu, d);
  if (st) return st;
  const int n = 30;
  std::fill(ke, ke + n * n, 0.0);
  double vol = 0.0;
  const double w = 1.0 / 24.0;
  std::vector<double> b(6 * n), tmp;
  for (int g = 0; g < 4; ++g) {
    double N[10], dn[10][3], dndx[10][3], det;
    tet10_shape(TET_PTS[g][0], TET_PTS[g][1], TET_PTS[g][2], N, dn);
    st = hex_dndx<10>(xyz, dn, dndx, &det);
    if (st) return st;
    if (det <= 0.0) return ERR_NEG_JACOBIAN;
    std::fill(b.begin(), b.end(), 0.0);
    fill_b3(b.data(), 10, dndx);
    gemm_bt_d_b(ke, n, b.data(), 6, d, w * det, tmp);
    vol += w * det;
  }
  *vol_out = vol;
  return OK;
}

// extra.rs:8-49: Gauss-Jordan with partial pivoting, singular below 1e-18
int invert_n(const std::vector<double>& a, int n, std::vector<double>& inv) {
  std::vector<double> m = a;
  inv.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) inv[(size_t)i * n + i] = 1.0;
  for (int k = 0; k < n; ++k) {
    int piv = k;
    double best = std::fabs(m[(size_t)k * n + k]);
    for (int i = k + 1; i < n; ++i) {
      const double v = std::fabs(m[(size_t)i * n + k]);
      if (v > best) {
        best = v;
        piv = i;
      }
    }
    if (best < 1e-18) return ERR_SINGULAR_JACOBIAN;  // "Kleine Matrix singulaer" (extra.rs:25)
    if (piv != k)
      for (int j = 0; j < n; ++j) {
        std::swap(m[(size_t)k * n + j], m[(size_t)piv * n + j]);
        std::swap(inv[(size_t)k * n + j], inv[(size_t)piv * n + j]);
      }
    const double d = m[(size_t)k * n + k];
    for (int j = 0; j < n; ++j) {
      m[(size_t)k * n + j] /= d;
      inv[(size_t)k * n + j] /= d;
    }
    for (int i = 0; i < n; ++i) {
      if (i == k) continue;
      const double f = m[(size_t)i * n + k];
      for (int j = 0; j < n; ++j) {
        m[(size_t)i * n + j] -= f * m[(size_t)k * n + j];
        inv[(size_t)i * n + j] -= f * inv[(size_t)k * n + j];
      }
    }
  }
  return OK;
}

// extra.rs:256-388: C3D8 with nine incompatible modes (Wilson-Taylor, modes
// mapped with the centre Jacobian), condensed statically
int hex8i_stiffness(const double* xyz, double e, double nu, double* kee, double* vol_out) {
  double d[36];
  int st = d_iso_3d(e, nu, d);
  if (st) return st;
  const int n = 24, ni = 9;
  std::fill(kee, kee + n * n, 0.0);
  std::vector<double> kea((size_t)n * ni, 0.0), kaa((size_t)ni * ni, 0.0);
  double vol = 0.0;
  double N0[8], dn0[8][3], dndx0[8][3], det0;
  hex8_shape(0.0, 0.0, 0.0, N0, dn0);
  st = hex_dndx<8>(xyz, dn0, dndx0, &det0);
  if (st) return st;
  if (det0 <= 0.0) return ERR_NEG_JACOBIAN;
  double j0[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int a = 0; a < 8; ++a)
    for (int p = 0; p < 3; ++p)
      for (int q = 0; q < 3; ++q) j0[q][p] += dn0[a][p] * xyz[3 * a + q];
  double inv0[3][3], dj;
  st = invert3(j0, inv0, &dj);
  if (st) return st;
  const double pts[2] = {-G2, G2};
  std::vector<double> be(6 * n), ba(6 * ni), tmp, tmp2(6 * ni);
  for (double xi : pts)
    for (double eta : pts)
      for (double zeta : pts) {
        double N[8], dn[8][3], dndx[8][3], det;
        hex8_shape(xi, eta, zeta, N, dn);
        st = hex_dndx<8>(xyz, dn, dndx, &det);
        if (st) return st;
        if (det <= 0.0) return ERR_NEG_JACOBIAN;
        std::fill(be.begin(), be.end(), 0.0);
        fill_b3(be.data(), 8, dndx);
        gemm_bt_d_b(kee, n, be.data(), 6, d, det, tmp);
        vol += det;
        std::fill(ba.begin(), ba.end(), 0.0);
        const double dparent[3][3] = {{-2.0 * xi, 0.0, 0.0}, {0.0, -2.0 * eta, 0.0}, {0.0, 0.0, -2.0 * zeta}};
        for (int m = 0; m < 3; ++m) {
          double g[3];
          for (int i = 0; i < 3; ++i)
            g[i] = inv0[0][i] * dparent[m][0] + inv0[1][i] * dparent[m][1] + inv0[2][i] * dparent[m][2];
          for (int dir = 0; dir < 3; ++dir) {
            const int col = m * 3 + dir;
            if (dir == 0) {
              ba[0 * ni + col] = g[0];
              ba[3 * ni + col] = g[1];
              ba[5 * ni + col] = g[2];
            } else if (dir == 1) {
              ba[1 * ni + col] = g[1];
              ba[3 * ni + col] = g[0];
              ba[4 * ni + col] = g[2];
            } else {
              ba[2 * ni + col] = g[2];
              ba[4 * ni + col] = g[1];
              ba[5 * ni + col] = g[0];
            }
          }
        }
        for (int i = 0; i < 6; ++i)
          for (int j = 0; j < ni; ++j) {
            double t = 0.0;
            for (int k = 0; k < 6; ++k) t += d[i * 6 + k] * ba[k * ni + j];
            tmp2[i * ni + j] = t;
          }
        for (int i = 0; i < ni; ++i)
          for (int j = 0; j < ni; ++j) {
            double t = 0.0;
            for (int k = 0; k < 6; ++k) t += ba[k * ni + i] * tmp2[k * ni + j];
            kaa[(size_t)i * ni + j] += det * t;
          }
        for (int i = 0; i < n; ++i)
          for (int j = 0; j < ni; ++j) {
            double t = 0.0;
            for (int k = 0; k < 6; ++k) t += be[k * n + i] * tmp2[k * ni + j];
            kea[(size_t)i * ni + j] += det * t;
          }
      }
  std::vector<double> kinv;
  st = invert_n(kaa, ni, kinv);
  if (st) return st;
  std::vector<double> t((size_t)ni * n);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < ni; ++i) {
      double x = 0.0;
      for (int k = 0; k < ni; ++k) x += kinv[(size_t)i * ni + k] * kea[(size_t)j * ni + k];
      t[(size_t)i * n + j] = x;
    }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double x = 0.0;
      for (int k = 0; k < ni; ++k) x += kea[(size_t)i * ni + k] * t[(size_t)k * n + j];
      kee[(size_t)i * n + j] -= x;
    }
  *vol_out = vol;
  return OK;
}

const double HOURGLASS[4][8] = {{1, -1, 1, -1, 1, -1, 1, -1},  // extra.rs:413-418
                                {1, 1, -1, -1, -1, -1, 1, 1},
                                {1, -1, -1, 1, -1, 1, 1, -1},
                                {-1, 1, -1, 1, 1, -1, 1, -1}};

// extra.rs:400-457: one-point C3D8 plus Flanagan-Belytschko hourglass stiffness
int hex8r_stiffness(const double* xyz, double e, double nu, double* ke, double* vol_out) {
  double d[36];
  int st = d_iso_3d(e, nu, d);
  if (st) return st;
  const int n = 24;
  std::fill(ke, ke + n * n, 0.0);
  double N[8], dn[8][3], dndx[8][3], det;
  hex8_shape(0.0, 0.0, 0.0, N, dn);
  st = hex_dndx<8>(xyz, dn, dndx, &det);
  if (st) return st;
  if (det <= 0.0) return ERR_NEG_JACOBIAN;
  const double vol = 8.0 * det;
  std::vector<double> b(6 * n, 0.0), tmp;
  fill_b3(b.data(), 8, dndx);
  gemm_bt_d_b(ke, n, b.data(), 6, d, vol, tmp);
  double gamma[4][8];
  for (int al = 0; al < 4; ++al) {
    double hx[3] = {0.0, 0.0, 0.0};
    for (int a = 0; a < 8; ++a)
      for (int j = 0; j < 3; ++j) hx[j] += HOURGLASS[al][a] * xyz[3 * a + j];
    for (int a = 0; a < 8; ++a) {
      double g = HOURGLASS[al][a];
      for (int j = 0; j < 3; ++j) g -= hx[j] * dndx[a][j];
      gamma[al][a] = g;
    }
  }
  const double mu = e / (2.0 * (1.0 + nu));
  const double coeff = 0.1 * mu * std::pow(vol, 1.0 / 3.0);
  for (int al = 0; al < 4; ++al) {
    double g2 = 0.0;
    for (int a = 0; a < 8; ++a) g2 += gamma[al][a] * gamma[al][a];
    if (g2 < 1e-30) continue;
    const double q = coeff / std::max(g2, 1e-30);
    for (int a = 0; a < 8; ++a)
      for (int bn = 0; bn < 8; ++bn) {
        const double v = q * gamma[al][a] * gamma[al][bn];
        for (int dir = 0; dir < 3; ++dir) ke[(3 * a + dir) * n + (3 * bn + dir)] += v;
      }
  }
  *vol_out = vol;
  return OK;
}

// extra.rs:64-87: linear wedge, triangle coordinates (xi, eta) x zeta
void wedge6_shape(double xi, double eta, double zeta, double n[6], double dn[6][3]) {
  const double l1 = xi, l2 = eta, l3 = 1.0 - xi - eta, zm = 0.5 * (1.0 - zeta), zp = 0.5 * (1.0 + zeta);
  n[0] = l1 * zm; n[1] = l2 * zm; n[2] = l3 * zm; n[3] = l1 * zp; n[4] = l2 * zp; n[5] = l3 * zp;
  const double t[6][3] = {{zm, 0.0, -0.5 * l1}, {0.0, zm, -0.5 * l2}, {-zm, -zm, -0.5 * l3},
                          {zp, 0.0, 0.5 * l1},  {0.0, zp, 0.5 * l2},  {-zp, -zp, 0.5 * l3}};
  for (int a = 0; a < 6; ++a)
    for (int p = 0; p < 3; ++p) dn[a][p] = t[a][p];
}

// extra.rs:701-756: quadratic wedge
void wedge15_shape(double xi, double eta, double zeta, double n[15], double dn[15][3]) {
  const double l1 = xi, l2 = eta, l3 = 1.0 - xi - eta, zm = 1.0 - zeta, zp = 1.0 + zeta;
  n[0] = 0.5 * l1 * zm * (2.0 * l1 - 2.0 - zeta);
  n[1] = 0.5 * l2 * zm * (2.0 * l2 - 2.0 - zeta);
  n[2] = 0.5 * l3 * zm * (2.0 * l3 - 2.0 - zeta);
  n[3] = 0.5 * l1 * zp * (2.0 * l1 - 2.0 + zeta);
  n[4] = 0.5 * l2 * zp * (2.0 * l2 - 2.0 + zeta);
  n[5] = 0.5 * l3 * zp * (2.0 * l3 - 2.0 + zeta);
  n[6] = 2.0 * l1 * l2 * zm;
  n[7] = 2.0 * l2 * l3 * zm;
  n[8] = 2.0 * l3 * l1 * zm;
  n[9] = 2.0 * l1 * l2 * zp;
  n[10] = 2.0 * l2 * l3 * zp;
  n[11] = 2.0 * l3 * l1 * zp;
  n[12] = l1 * (1.0 - zeta * zeta);
  n[13] = l2 * (1.0 - zeta * zeta);
  n[14] = l3 * (1.0 - zeta * zeta);
  const double d1b = 0.5 * zm * (4.0 * l1 - 2.0 - zeta), d2b = 0.5 * zm * (4.0 * l2 - 2.0 - zeta),
               d3b = 0.5 * zm * (4.0 * l3 - 2.0 - zeta);
  const double d1t = 0.5 * zp * (4.0 * l1 - 2.0 + zeta), d2t = 0.5 * zp * (4.0 * l2 - 2.0 + zeta),
               d3t = 0.5 * zp * (4.0 * l3 - 2.0 + zeta);
  const double o = 1.0 - zeta * zeta;
  const double t[15][3] = {{d1b, 0.0, -0.5 * l1 * (2.0 * l1 - 1.0 - 2.0 * zeta)},
                           {0.0, d2b, -0.5 * l2 * (2.0 * l2 - 1.0 - 2.0 * zeta)},
                           {-d3b, -d3b, -0.5 * l3 * (2.0 * l3 - 1.0 - 2.0 * zeta)},
                           {d1t, 0.0, 0.5 * l1 * (2.0 * l1 - 1.0 + 2.0 * zeta)},
                           {0.0, d2t, 0.5 * l2 * (2.0 * l2 - 1.0 + 2.0 * zeta)},
                           {-d3t, -d3t, 0.5 * l3 * (2.0 * l3 - 1.0 + 2.0 * zeta)},
                           {2.0 * l2 * zm, 2.0 * l1 * zm, -2.0 * l1 * l2},
                           {-2.0 * l2 * zm, 2.0 * (l3 - l2) * zm, -2.0 * l2 * l3},
                           {2.0 * (l3 - l1) * zm, -2.0 * l1 * zm, -2.0 * l3 * l1},
                           {2.0 * l2 * zp, 2.0 * l1 * zp, 2.0 * l1 * l2},
                           {-2.0 * l2 * zp, 2.0 * (l3 - l2) * zp, 2.0 * l2 * l3},
                           {2.0 * (l3 - l1) * zp, -2.0 * l1 * zp, 2.0 * l3 * l1},
                           {o, 0.0, -2.0 * zeta * l1},
                           {0.0, o, -2.0 * zeta * l2},
                           {-o, -o, -2.0 * zeta * l3}};
  for (int a = 0; a < 15; ++a)
    for (int p = 0; p < 3; ++p) dn[a][p] = t[a][p];
}

const double WTRI[3][2] = {{1.0 / 6.0, 1.0 / 6.0}, {2.0 / 3.0, 1.0 / 6.0}, {1.0 / 6.0, 2.0 / 3.0}};  // extra.rs:114

// extra.rs:109-132 (C3D6: 3 triangle points x 2 in zeta, w = 1/6) and 783-819
// (C3D15: 3 triangle points x 3 in zeta, w = W3 / 6)
template <int NN>
int wedge_stiffness(const double* xyz, double e, double nu, double* ke, double* vol_out) {
  double d[36];
  int st = d_iso_3d(e, nu, d);
  if (st) return st;
  const int n = 3 * NN;
  std::fill(ke, ke + n * n, 0.0);
  double vol = 0.0;
  std::vector<double> b(6 * n), tmp;
  const int nz = NN == 6 ? 2 : 3;
  for (int t = 0; t < 3; ++t)
    for (int k = 0; k < nz; ++k) {
      const double zeta = NN == 6 ? (k == 0 ? -G2 : G2) : G3[k];
      const double w0 = NN == 6 ? 1.0 / 6.0 : (1.0 / 6.0) * W3[k];
      double N[NN], dn[NN][3], dndx[NN][3], det;
      if (NN == 6)
        wedge6_shape(WTRI[t][0], WTRI[t][1], zeta, (double*)N, (double(*)[3])dn);
      else
        wedge15_shape(WTRI[t][0], WTRI[t][1], zeta, (double*)N, (double(*)[3])dn);
      st = hex_dndx<NN>(xyz, dn, dndx, &det);
      if (st) return st;
      if (det <= 0.0) return ERR_NEG_JACOBIAN;
      const double w = det * w0;
      std::fill(b.begin(), b.end(), 0.0);
      fill_b3(b.data(), NN, dndx);
      gemm_bt_d_b(ke, n, b.data(), 6, d, w, tmp);
      vol += w;
    }
  *vol_out = vol;
  return OK;
}

// nn = 8: reduced 0 = C3D8, 1 = C3D8R, 2 = C3D8I; nn = 20: reduced 1 = C3D20R
int element_ke(int nn, const double* xyz, double e, double nu, int reduced, double* ke, double* vol) {
  if (nn == 8 && reduced == 1) return hex8r_stiffness(xyz, e, nu, ke, vol);
  if (nn == 8 && reduced == 2) return hex8i_stiffness(xyz, e, nu, ke, vol);
  if (nn == 4) return tet4_stiffness(xyz, e, nu, ke, vol);
  if (nn == 10) return tet10_stiffness(xyz, e, nu, ke, vol);
  if (nn == 6) return wedge_stiffness<6>(xyz, e, nu, ke, vol);
  if (nn == 15) return wedge_stiffness<15>(xyz, e, nu, ke, vol);
  if (nn == 8) {
    double d[36];
    int st = d_iso_3d(e, nu, d);
    if (st) return st;
    return hex8_stiffness_d(xyz, d, ke, vol);
  }
  if (nn == 20) return hex20_stiffness(xyz, e, nu, reduced != 0, ke, vol);
  return ERR_INVALID_ARG;
}

// A triplet as the reference stores it: (usize, usize, f64).
struct Trip {
  uint64_t i, j;
  double v;
};

// linalg.rs:3-8
struct Csr {
  size_t n = 0;
  std::vector<uint64_t> indptr, indices;
  std::vector<double> data;
};

// linalg.rs:10-38: drop out-of-range and zero entries, stable sort by (i,j),
// sum duplicates in input order (explicit zero sums are kept).
void csr_from_triplets(size_t n, std::vector<Trip>& trips, Csr& out) {
  trips.erase(std::remove_if(trips.begin(), trips.end(),
                             [n](const Trip& t) { return !(t.i < n && t.j < n && std::fabs(t.v) > 0.0); }),
              trips.end());
  std::stable_sort(trips.begin(), trips.end(), [](const Trip& a, const Trip& b) {
    return a.i != b.i ? a.i < b.i : a.j < b.j;
  });
  out.n = n;
  out.indptr.assign(n + 1, 0);
  out.indices.clear();
  out.data.clear();
  out.indices.reserve(trips.size());
  out.data.reserve(trips.size());
  size_t k = 0;
  while (k < trips.size()) {
    uint64_t i = trips[k].i, j = trips[k].j;
    double v = 0.0;
    while (k < trips.size() && trips[k].i == i && trips[k].j == j) {
      v += trips[k].v;
      ++k;
    }
    out.indices.push_back(j);
    out.data.push_back(v);
    out.indptr[i + 1] += 1;
  }
  for (size_t i = 0; i < n; ++i) out.indptr[i + 1] += out.indptr[i];
}

// linalg.rs:41-50 (serial as written; nthreads > 1 splits rows over OpenMP,
// each row is still summed in column order so the result is unchanged).
void matvec(const Csr& a, const double* x, double* y, int nthreads) {
  const int64_t n = (int64_t)a.n;
#pragma omp parallel for schedule(static) num_threads(nthreads) if (nthreads > 1)
  for (int64_t i = 0; i < n; ++i) {
    double s = 0.0;
    for (uint64_t k = a.indptr[i]; k < a.indptr[i + 1]; ++k) s += a.data[k] * x[a.indices[k]];
    y[i] = s;
  }
}

// linalg.rs:52-63
std::vector<double> csr_diag(const Csr& a) {
  std::vector<double> d(a.n, 0.0);
  for (size_t i = 0; i < a.n; ++i)
    for (uint64_t k = a.indptr[i]; k < a.indptr[i + 1]; ++k)
      if (a.indices[k] == i) {
        d[i] = a.data[k];
        break;
      }
  return d;
}

double dotp(const double* a, const double* b, int64_t n, int nthreads) {
  if (nthreads <= 1) {
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
  }
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static) num_threads(nthreads)
  for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

// linalg.rs:199-259.  nthreads == 1 reproduces the serial reference order.
int pcg(const Csr& a, const double* b, double tol, size_t max_iter, int nthreads, double* x,
        size_t* iters_out, double* residual_out) {
  const int64_t n = (int64_t)a.n;
  std::fill(x, x + n, 0.0);
  std::vector<double> r(b, b + n);
  double bnorm = 0.0;
  for (int64_t i = 0; i < n; ++i) bnorm += b[i] * b[i];
  bnorm = std::sqrt(bnorm);
  if (bnorm < 1e-30) {
    *iters_out = 0;
    *residual_out = 0.0;
    return OK;
  }
  std::vector<double> diag = csr_diag(a);
  std::vector<double> z(n), p, ap(n);
  for (int64_t i = 0; i < n; ++i) z[i] = r[i] / (std::fabs(diag[i]) > 1e-30 ? diag[i] : 1.0);
  p = z;
  double rz = dotp(r.data(), z.data(), n, nthreads);
  size_t iters = 0;
  double residual = bnorm;
  for (size_t it = 0; it < max_iter; ++it) {
    iters = it + 1;
    matvec(a, p.data(), ap.data(), nthreads);
    double pap = dotp(p.data(), ap.data(), n, nthreads);
    if (std::fabs(pap) < 1e-30) {
      *iters_out = iters;
      *residual_out = residual;
      return ERR_ZERO_PIVOT;
    }
    double alpha = rz / pap;
#pragma omp parallel for schedule(static) num_threads(nthreads) if (nthreads > 1)
    for (int64_t i = 0; i < n; ++i) {
      x[i] += alpha * p[i];
      r[i] -= alpha * ap[i];
    }
    residual = std::sqrt(dotp(r.data(), r.data(), n, nthreads));
    if (residual <= tol * bnorm) break;
#pragma omp parallel for schedule(static) num_threads(nthreads) if (nthreads > 1)
    for (int64_t i = 0; i < n; ++i) z[i] = r[i] / (std::fabs(diag[i]) > 1e-30 ? diag[i] : 1.0);
    double rz_new = dotp(r.data(), z.data(), n, nthreads);
    double beta = rz_new / rz;
#pragma omp parallel for schedule(static) num_threads(nthreads) if (nthreads > 1)
    for (int64_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    rz = rz_new;
  }
  *iters_out = iters;
  *residual_out = residual;
  if (residual > tol * bnorm * 10.0) return ERR_NOT_CONVERGED;
  return OK;
}

// linalg.rs:78-117
int chol_solve(double* a, size_t n, const double* b, double* x) {
  for (size_t i = 0; i < n; ++i)
    for (size_t j = 0; j <= i; ++j) {
      double s = a[i * n + j];
      for (size_t k = 0; k < j; ++k) s -= a[i * n + k] * a[j * n + k];
      if (i == j) {
        if (s < 0.0) return ERR_INDEFINITE;
        if (s <= 1e-30) return ERR_SINGULAR;
        a[i * n + i] = std::sqrt(s);
      } else {
        a[i * n + j] = s / a[j * n + j];
      }
    }
  std::vector<double> y(n);
  for (size_t i = 0; i < n; ++i) {
    double s = b[i];
    for (size_t k = 0; k < i; ++k) s -= a[i * n + k] * y[k];
    y[i] = s / a[i * n + i];
  }
  for (size_t ii = n; ii-- > 0;) {
    double s = y[ii];
    for (size_t k = ii + 1; k < n; ++k) s -= a[k * n + ii] * x[k];
    x[ii] = s / a[ii * n + ii];
  }
  return OK;
}

// linalg.rs:268-278
double residual_of(const Csr& a, const double* x, const double* b) {
  std::vector<double> ax(a.n);
  matvec(a, x, ax.data(), 1);
  double s = 0.0;
  for (size_t i = 0; i < a.n; ++i) {
    double d = ax[i] - b[i];
    s += d * d;
  }
  return std::sqrt(s);
}

// elem.rs:725-742
void sigma_from_b(const double* b, int nrow, int n, const double* d, const double* ue, double* sig) {
  double eps[6];
  for (int r = 0; r < nrow; ++r) {
    double t = 0.0;
    for (int j = 0; j < n; ++j) t += b[r * n + j] * ue[j];
    eps[r] = t;
  }
  for (int r = 0; r < nrow; ++r) {
    double t = 0.0;
    for (int k = 0; k < nrow; ++k) t += d[r * nrow + k] * eps[k];
    sig[r] = t;
  }
}

// elem.rs:744-779: Gauss-point stresses at HEX_XI * G2, extrapolated with the
// trilinear shapes evaluated at HEX_XI * sqrt(3)
int hex8_nodal_stress(const double* xyz, const double* ue, double e, double nu, double out[8][6]) {
  double d[36];
  int st = d_iso_3d(e, nu, d);
  if (st) return st;
  const int n = 24;
  double gsig[8][6];
  std::vector<double> b(6 * n);
  for (int i = 0; i < 8; ++i) {
    double N[8], dn[8][3], dndx[8][3], det;
    hex8_shape(HEX_XI[i][0] * G2, HEX_XI[i][1] * G2, HEX_XI[i][2] * G2, N, dn);
    st = hex_dndx<8>(xyz, dn, dndx, &det);
    if (st) return st;
    std::fill(b.begin(), b.end(), 0.0);
    fill_b3(b.data(), 8, dndx);
    sigma_from_b(b.data(), 6, n, d, ue, gsig[i]);
  }
  const double s3 = std::sqrt(3.0);
  for (int a = 0; a < 8; ++a) {
    double N[8], dn[8][3];
    hex8_shape(HEX_XI[a][0] * s3, HEX_XI[a][1] * s3, HEX_XI[a][2] * s3, N, dn);
    for (int c = 0; c < 6; ++c) {
      double v = 0.0;
      for (int g = 0; g < 8; ++g) v += N[g] * gsig[g][c];
      out[a][c] = v;
    }
  }
  return OK;
}

// quadratic.rs:227-244
void lagrange1d(const double* pts, int n, double x, double* w) {
  for (int i = 0; i < n; ++i) {
    w[i] = 1.0;
    for (int j = 0; j < n; ++j) {
      if (i == j) continue;
      w[i] *= (x - pts[j]) / (pts[i] - pts[j]);
    }
  }
}

// quadratic.rs:148-171 + hex20_extrapolate 205-225
int hex20_nodal_stress(const double* xyz, const double* ue, double e, double nu, bool reduced, double out[20][6]) {
  double d[36];
  int st = d_iso_3d(e, nu, d);
  if (st) return st;
  const int n = 60;
  std::vector<double> gp, b(6 * n);
  hex_gauss(reduced, gp);
  const int ng = (int)gp.size() / 4;
  std::vector<double> gsig((size_t)ng * 6);
  for (int g = 0; g < ng; ++g) {
    double N[20], dn[20][3], dndx[20][3], det;
    hex20_shape(gp[4 * g], gp[4 * g + 1], gp[4 * g + 2], N, dn);
    st = hex_dndx<20>(xyz, dn, dndx, &det);
    if (st) return st;
    std::fill(b.begin(), b.end(), 0.0);
    fill_b3(b.data(), 20, dndx);
    sigma_from_b(b.data(), 6, n, d, ue, &gsig[6 * g]);
  }
  const double p2[2] = {-G2, G2};
  const double* pts = reduced ? p2 : G3;
  const int n1 = reduced ? 2 : 3;
  for (int a = 0; a < 20; ++a) {
    double lx[3], ly[3], lz[3];
    lagrange1d(pts, n1, HEX20_XI[a][0], lx);
    lagrange1d(pts, n1, HEX20_XI[a][1], ly);
    lagrange1d(pts, n1, HEX20_XI[a][2], lz);
    for (int c = 0; c < 6; ++c) out[a][c] = 0.0;
    int idx = 0;
    for (int i = 0; i < n1; ++i)
      for (int j = 0; j < n1; ++j)
        for (int k = 0; k < n1; ++k, ++idx) {
          const double w = lx[i] * ly[j] * lz[k];
          for (int c = 0; c < 6; ++c) out[a][c] += w * gsig[6 * idx + c];
        }
  }
  return OK;
}

// extra.rs:460-472: the centre stress at all eight nodes
int hex8r_nodal_stress(const double* xyz, const double* ue, double e, double nu, double out[20][6]) {
  double d[36];
  int st = d_iso_3d(e, nu, d);
  if (st) return st;
  double N[8], dn[8][3], dndx[8][3], det;
  hex8_shape(0.0, 0.0, 0.0, N, dn);
  st = hex_dndx<8>(xyz, dn, dndx, &det);
  if (st) return st;
  const int n = 24;
  std::vector<double> b(6 * n, 0.0);
  fill_b3(b.data(), 8, dndx);
  double sig[6];
  sigma_from_b(b.data(), 6, n, d, ue, sig);
  for (int a = 0; a < 8; ++a)
    for (int c = 0; c < 6; ++c) out[a][c] = sig[c];
  return OK;
}

// extra.rs:134-154 / 821-850: stresses evaluated at the wedge's nodes
template <int NN>
int wedge_nodal_stress(const double* xyz, const double* ue, double e, double nu, double out[20][6]) {
  double d[36];
  int st = d_iso_3d(e, nu, d);
  if (st) return st;
  const double pts[15][3] = {{1, 0, -1}, {0, 1, -1}, {0, 0, -1}, {1, 0, 1},    {0, 1, 1},
                             {0, 0, 1},  {0.5, 0.5, -1}, {0, 0.5, -1}, {0.5, 0, -1}, {0.5, 0.5, 1},
                             {0, 0.5, 1}, {0.5, 0, 1},  {1, 0, 0},   {0, 1, 0},    {0, 0, 0}};
  const int n = 3 * NN;
  std::vector<double> b(6 * n);
  for (int a = 0; a < NN; ++a) {
    double N[NN], dn[NN][3], dndx[NN][3], det;
    if (NN == 6)
      wedge6_shape(pts[a][0], pts[a][1], pts[a][2], (double*)N, (double(*)[3])dn);
    else
      wedge15_shape(pts[a][0], pts[a][1], pts[a][2], (double*)N, (double(*)[3])dn);
    st = hex_dndx<NN>(xyz, dn, dndx, &det);
    if (st) return st;
    std::fill(b.begin(), b.end(), 0.0);
    fill_b3(b.data(), NN, dndx);
    sigma_from_b(b.data(), 6, n, d, ue, out[a]);
  }
  return OK;
}

// elem.rs:781-795: one constant stress for all four nodes
int tet4_nodal_stress(const double* xyz, const double* ue, double e, double nu, double out[20][6]) {
  double dndx[4][3], det;
  int st = tet4_dndx(xyz, dndx, &det);
  if (st) return st;
  double d[36];
  st = d_iso_3d(e, nu, d);
  if (st) return st;
  const int n = 12;
  std::vector<double> b(6 * n, 0.0);
  fill_b3(b.data(), 4, dndx);
  double sig[6];
  sigma_from_b(b.data(), 6, n, d, ue, sig);
  for (int a = 0; a < 4; ++a)
    for (int c = 0; c < 6; ++c) out[a][c] = sig[c];
  return OK;
}

// quadratic.rs:678-702: stresses evaluated at the ten nodes
int tet10_nodal_stress(const double* xyz, const double* ue, double e, double nu, double out[20][6]) {
  double d[36];
  int st = d_iso_3d(e, nu, d);
  if (st) return st;
  const double rst[10][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0.5, 0, 0},
                             {0.5, 0.5, 0}, {0, 0.5, 0}, {0, 0, 0.5}, {0.5, 0, 0.5}, {0, 0.5, 0.5}};
  const int n = 30;
  std::vector<double> b(6 * n);
  for (int a = 0; a < 10; ++a) {
    double N[10], dn[10][3], dndx[10][3], det;
    tet10_shape(rst[a][0], rst[a][1], rst[a][2], N, dn);
    st = hex_dndx<10>(xyz, dn, dndx, &det);
    if (st) return st;
    std::fill(b.begin(), b.end(), 0.0);
    fill_b3(b.data(), 10, dndx);
    sigma_from_b(b.data(), 6, n, d, ue, out[a]);
  }
  return OK;
}

// elem.rs:651-660
double von_mises(const double* s) {
  const double sx = s[0], sy = s[1], sz = s[2], txy = s[3], tyz = s[4], tzx = s[5];
  return std::sqrt(0.5 * ((sx - sy) * (sx - sy) + (sy - sz) * (sy - sz) + (sz - sx) * (sz - sx)) +
                   3.0 * (txy * txy + tyz * tyz + tzx * tzx));
}

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

extern "C" {

int or_version() { return 1; }

void or_hex8_shape(double xi, double eta, double zeta, double* n, double* dn) {
  hex8_shape(xi, eta, zeta, n, reinterpret_cast<double(*)[3]>(dn));
}
void or_hex20_shape(double xi, double eta, double zeta, double* n, double* dn) {
  hex20_shape(xi, eta, zeta, n, reinterpret_cast<double(*)[3]>(dn));
}
void or_quad8_shape(double xi, double eta, double* n, double* dn) {
  quad8_shape(xi, eta, n, reinterpret_cast<double(*)[2]>(dn));
}
int or_invert3(const double* a9, double* inv9, double* det) {
  double a[3][3], b[3][3];
  std::memcpy(a, a9, sizeof(a));
  int st = invert3(a, b, det);
  if (st == OK) std::memcpy(inv9, b, sizeof(b));
  return st;
}
int or_d_iso_3d(double e, double nu, double* d36) { return d_iso_3d(e, nu, d36); }

// element_ke (elem.rs:344-375 Hex8 arm, elem.rs:487-495 Hex20 arm) for one element.
int or_element_ke(int nn, const double* xyz, double e, double nu, int reduced, double* ke, double* vol) {
  return element_ke(nn, xyz, e, nu, reduced, ke, vol);
}

namespace {
// extra.rs:197-213: flat triangle, a third of -p * area vector per node
void tri_face_load(double* fe, const double* xyz, const int idx[3], double p) {
  const double* a = xyz + 3 * idx[0];
  const double* b = xyz + 3 * idx[1];
  const double* c = xyz + 3 * idx[2];
  const double ux[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
  const double vx[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
  const double nx = ux[1] * vx[2] - ux[2] * vx[1];
  const double ny = ux[2] * vx[0] - ux[0] * vx[2];
  const double nz = ux[0] * vx[1] - ux[1] * vx[0];
  const double sc = -p * 0.5 / 3.0;
  for (int k = 0; k < 3; ++k) {
    fe[3 * idx[k]] += sc * nx;
    fe[3 * idx[k] + 1] += sc * ny;
    fe[3 * idx[k] + 2] += sc * nz;
  }
}

// extra.rs:215-253: bilinear quadrilateral, 2x2 Gauss
void quad_face_load(double* fe, const double* xyz, const int idx[4], double p) {
  const double pts[2] = {-G2, G2};
  for (double xi : pts)
    for (double eta : pts) {
      double n[4], dnxi[4], dneta[4];
      for (int i = 0; i < 4; ++i) {
        const double x = QUAD_XI[i][0], e = QUAD_XI[i][1];
        n[i] = 0.25 * (1.0 + x * xi) * (1.0 + e * eta);
        dnxi[i] = 0.25 * x * (1.0 + e * eta);
        dneta[i] = 0.25 * e * (1.0 + x * xi);
      }
      double rxi[3] = {0, 0, 0}, reta[3] = {0, 0, 0};
      for (int a = 0; a < 4; ++a)
        for (int k = 0; k < 3; ++k) {
          rxi[k] += dnxi[a] * xyz[3 * idx[a] + k];
          reta[k] += dneta[a] * xyz[3 * idx[a] + k];
        }
      const double nx = rxi[1] * reta[2] - rxi[2] * reta[1];
      const double ny = rxi[2] * reta[0] - rxi[0] * reta[2];
      const double nz = rxi[0] * reta[1] - rxi[1] * reta[0];
      for (int a = 0; a < 4; ++a) {
        fe[3 * idx[a]] += -p * n[a] * nx;
        fe[3 * idx[a] + 1] += -p * n[a] * ny;
        fe[3 * idx[a] + 2] += -p * n[a] * nz;
      }
    }
}

// extra.rs:882-924: quadratic triangle, 3 points, w = 1/6
void tri6_face_load(double* fe, const double* xyz, const int idx[6], double p) {
  const double w0 = 1.0 / 6.0;
  for (int g = 0; g < 3; ++g) {
    const double l1 = WTRI[g][0], l2 = WTRI[g][1], l3 = 1.0 - l1 - l2;
    const double ns[6] = {l1 * (2.0 * l1 - 1.0), l2 * (2.0 * l2 - 1.0), l3 * (2.0 * l3 - 1.0),
                          4.0 * l1 * l2,         4.0 * l2 * l3,         4.0 * l3 * l1};
    const double dn1[6] = {4.0 * l1 - 1.0, 0.0, -(4.0 * l3 - 1.0), 4.0 * l2, -4.0 * l2, 4.0 * (l3 - l1)};
    const double dn2[6] = {0.0, 4.0 * l2 - 1.0, -(4.0 * l3 - 1.0), 4.0 * l1, 4.0 * (l3 - l2), -4.0 * l1};
    double rxi[3] = {0, 0, 0}, reta[3] = {0, 0, 0};
    for (int a = 0; a < 6; ++a)
      for (int k = 0; k < 3; ++k) {
        rxi[k] += dn1[a] * xyz[3 * idx[a] + k];
        reta[k] += dn2[a] * xyz[3 * idx[a] + k];
      }
    const double nx = rxi[1] * reta[2] - rxi[2] * reta[1];
    const double ny = rxi[2] * reta[0] - rxi[0] * reta[2];
    const double nz = rxi[0] * reta[1] - rxi[1] * reta[0];
    for (int a = 0; a < 6; ++a) {
      fe[3 * idx[a]] += -p * ns[a] * nx * w0;
      fe[3 * idx[a] + 1] += -p * ns[a] * ny * w0;
      fe[3 * idx[a] + 2] += -p * ns[a] * nz * w0;
    }
  }
}

// extra.rs:926-954: serendipity quadrilateral, 3x3 Gauss
void quad8_face_load(double* fe, const double* xyz, const int idx[8], double p) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      const double w = W3[i] * W3[j];
      double ns[8], dn[8][2];
      quad8_shape(G3[i], G3[j], ns, dn);
      double rxi[3] = {0, 0, 0}, reta[3] = {0, 0, 0};
      for (int a = 0; a < 8; ++a)
        for (int k = 0; k < 3; ++k) {
          rxi[k] += dn[a][0] * xyz[3 * idx[a] + k];
          reta[k] += dn[a][1] * xyz[3 * idx[a] + k];
        }
      const double nx = rxi[1] * reta[2] - rxi[2] * reta[1];
      const double ny = rxi[2] * reta[0] - rxi[0] * reta[2];
      const double nz = rxi[0] * reta[1] - rxi[1] * reta[0];
      for (int a = 0; a < 8; ++a) {
        fe[3 * idx[a]] += -p * ns[a] * nx * w;
        fe[3 * idx[a] + 1] += -p * ns[a] * ny * w;
        fe[3 * idx[a] + 2] += -p * ns[a] * nz * w;
      }
    }
}

// extra.rs:184-195 and 869-880
int wedge_face_pressure(int nn, const double* xyz, int face, double p, double* fe) {
  std::fill(fe, fe + 3 * nn, 0.0);
  if (nn == 6) {
    static const int t1[3] = {0, 1, 2}, t2[3] = {3, 5, 4};
    static const int q[3][4] = {{0, 1, 4, 3}, {1, 2, 5, 4}, {2, 0, 3, 5}};
    if (face == 1) tri_face_load(fe, xyz, t1, p);
    else if (face == 2) tri_face_load(fe, xyz, t2, p);
    else if (face >= 3 && face <= 5) quad_face_load(fe, xyz, q[face - 3], p);
    else return ERR_INVALID_ARG;
    return OK;
  }
  static const int t1[6] = {0, 1, 2, 6, 7, 8}, t2[6] = {3, 5, 4, 11, 10, 9};
  static const int q[3][8] = {{0, 1, 4, 3, 6, 13, 9, 12}, {1, 2, 5, 4, 7, 14, 10, 13}, {2, 0, 3, 5, 8, 12, 11, 14}};
  if (face == 1) tri6_face_load(fe, xyz, t1, p);
  else if (face == 2) tri6_face_load(fe, xyz, t2, p);
  else if (face >= 3 && face <= 5) quad8_face_load(fe, xyz, q[face - 3], p);
  else return ERR_INVALID_ARG;
  return OK;
}
}  // namespace

int or_face_pressure(int nn, const double* xyz, int face, double p, double* fe) {
  if (nn == 6 || nn == 15) return wedge_face_pressure(nn, xyz, face, p, fe);
  if (nn == 8) return hex8_face_pressure(xyz, face, p, fe);
  if (nn == 20) return hex20_face_pressure(xyz, face, p, fe);
  if (nn == 4 || nn == 10) {  // apply_pressure has no tetrahedron arm (analysis.rs:1447): no load
    std::fill(fe, fe + 3 * nn, 0.0);
    return OK;
  }
  return ERR_INVALID_ARG;
}

// Consistent nodal forces of a list of face pressures, scattered into f_full
// in list order (analysis.rs:723-755 -> apply_pressure 1365-1396 -> scatter_fe
// 1546-1553).  Returns the index of the first failing load in *bad.
int or_face_loads(int64_t n_nodes, const double* coords, int nn, const int32_t* conn, int64_t n_loads,
                  const int64_t* elem, const int32_t* face, const double* p, double* f_full, int64_t* bad) {
  double xyz[60], fe[60];
  for (int64_t k = 0; k < n_loads; ++k) {
    const int32_t* c = conn + elem[k] * nn;
    for (int a = 0; a < nn; ++a)
      for (int q = 0; q < 3; ++q) xyz[3 * a + q] = coords[3 * (int64_t)c[a] + q];
    int st = or_face_pressure(nn, xyz, face[k], p[k], fe);
    if (st) {
      *bad = k;
      return st;
    }
    for (int a = 0; a < nn; ++a)
      for (int d = 0; d < 3; ++d) f_full[3 * (int64_t)c[a] + d] += fe[3 * a + d];
  }
  (void)n_nodes;
  return OK;
}

// Sparse-matrix handle held by the Python wrapper.
struct OrCsr {
  Csr csr;
};

// solve_linear (analysis.rs:548-1035) for a pure C3D8 / C3D20 isotropic model
// with single-point constraints, restricted to the linear *STATIC step:
//   prescribed = BCs in input order, last wins            (analysis.rs:556-565)
//   isolated nodes pinned                                  (analysis.rs:2283-2330)
//   element loop -> element_ke -> push nonzero triplets    (analysis.rs:574-668)
//   AUTOSPC null-diagonal pin                              (analysis.rs:2164-2228)
//   DofMap::build / reduce                                 (constraint.rs:26-172)
//   solve_kff: csr_from_triplets, then dense Cholesky (solver=1) or PCG
//   (solver=2) with tol, max_iter max(4n,200) when max_iter <= 0 (linalg.rs:311-404)
//   reconstruct                                            (constraint.rs:207-217)
// The reactions K u - f over the raw triplets (analysis.rs:1027-1035) go to rf_full.
// info[0..12] = n_free, nnz(K_ff CSR), iters, residual, t_assembly, t_reduce,
//               t_csr, t_solve, t_total, n_triplets, bnorm, first bad element
int or_solve_static(int64_t n_nodes, const double* coords, int nn, int reduced, int64_t n_elem,
                    const int32_t* conn, const double* e_elem, double nu, int64_t n_bc,
                    const int64_t* bc_dof, const double* bc_val, const double* f_in, int solver,
                    double tol, int64_t max_iter, int nthreads, int autospc, double* u_full,
                    double* rf_full, double* info, OrCsr** csr_out, double* rhs_out) {
  const double t0 = now_s();
  const int64_t ndof = 3 * n_nodes;
  for (int i = 0; i < 12; ++i) info[i] = 0.0;
  info[11] = -1;
  if (ndof == 0) return ERR_INVALID_ARG;
  // prescribed map: last BC wins; keep insertion semantics of a HashMap
  std::vector<char> is_presc(ndof, 0);
  std::vector<double> presc_val(ndof, 0.0);
  for (int64_t k = 0; k < n_bc; ++k) {
    int64_t d = bc_dof[k];
    if (d < 0 || d >= ndof) return ERR_INVALID_ARG;
    is_presc[d] = 1;
    presc_val[d] = bc_val[k];
  }
  if (autospc) {  // isolated nodes: all dofs pinned (or_insert: keeps an existing BC)
    std::vector<char> attached(n_nodes, 0);
    for (int64_t e = 0; e < n_elem; ++e)
      for (int a = 0; a < nn; ++a) attached[conn[e * nn + a]] = 1;
    for (int64_t ni = 0; ni < n_nodes; ++ni)
      if (!attached[ni])
        for (int d = 0; d < 3; ++d)
          if (!is_presc[3 * ni + d]) {
            is_presc[3 * ni + d] = 1;
            presc_val[3 * ni + d] = 0.0;
          }
  }
  // element loop
  std::vector<Trip> trips;
  trips.reserve((size_t)n_elem * (size_t)(9 * nn * nn));
  const int m = 3 * nn;
  std::vector<double> ke((size_t)m * m);
  double xyz[60], vol;
  for (int64_t e = 0; e < n_elem; ++e) {
    const int32_t* c = conn + e * nn;
    for (int a = 0; a < nn; ++a)
      for (int q = 0; q < 3; ++q) xyz[3 * a + q] = coords[3 * (int64_t)c[a] + q];
    int st = element_ke(nn, xyz, e_elem[e], nu, reduced, ke.data(), &vol);
    if (st) {
      info[11] = (double)e;
      return st;
    }
    for (int i = 0; i < m; ++i) {
      uint64_t gi = 3 * (uint64_t)c[i / 3] + (uint64_t)(i % 3);
      for (int j = 0; j < m; ++j) {
        double v = ke[(size_t)i * m + j];
        if (std::fabs(v) > 0.0) trips.push_back({gi, 3 * (uint64_t)c[j / 3] + (uint64_t)(j % 3), v});
      }
    }
  }
  const double t1 = now_s();
  std::vector<double> f_full(f_in, f_in + ndof);
  if (autospc) {  // analysis.rs:2208-2227
    std::vector<double> dg(ndof, 0.0);
    for (const Trip& t : trips)
      if (t.i == t.j) dg[t.i] += t.v;
    double max_d = 0.0;
    for (double v : dg) max_d = std::max(max_d, std::fabs(v));
    if (max_d >= 1e-30) {
      double tl = max_d * 1e-14;
      for (int64_t i = 0; i < ndof; ++i)
        if (!is_presc[i] && std::fabs(dg[i]) <= tl) {
          is_presc[i] = 1;
          presc_val[i] = 0.0;
        }
    }
  }
  // DofMap::build, prescribed subset (constraint.rs:26-136)
  std::vector<int64_t> ind_of(ndof, -1);
  int64_t n_ind = 0;
  for (int64_t d = 0; d < ndof; ++d)
    if (!is_presc[d]) ind_of[d] = n_ind++;
  bool any_presc = false;
  for (int64_t d = 0; d < ndof; ++d) any_presc |= is_presc[d] != 0;
  if (n_ind == 0 && !any_presc) return ERR_NO_FREE_DOF;
  std::vector<double> u0(ndof, 0.0);
  for (int64_t d = 0; d < ndof; ++d)
    if (is_presc[d]) u0[d] = presc_val[d];
  // DofMap::reduce (constraint.rs:138-172): t_row[d] = [(ind_of[d], 1.0)] for free d.
  std::vector<double> rhs(n_ind, 0.0);
  for (int64_t i = 0; i < ndof; ++i) {
    double fi = f_full[i];
    if (std::fabs(fi) == 0.0) continue;
    if (ind_of[i] >= 0) rhs[ind_of[i]] += 1.0 * fi;
  }
  std::vector<Trip> ff;
  ff.reserve(trips.size());
  for (const Trip& t : trips) {
    if (t.i >= (uint64_t)ndof || t.j >= (uint64_t)ndof || std::fabs(t.v) == 0.0) continue;
    double u0j = u0[t.j];
    int64_t a = ind_of[t.i];
    if (a < 0) continue;
    if (std::fabs(u0j) > 0.0) rhs[a] -= t.v * 1.0 * u0j;
    int64_t b = ind_of[t.j];
    if (b >= 0) ff.push_back({(uint64_t)a, (uint64_t)b, t.v * 1.0 * 1.0});
  }
  const double t2 = now_s();
  info[0] = (double)n_ind;
  info[9] = (double)ff.size();
  std::vector<double> u(ndof);
  if (n_ind == 0) {
    u = u0;
  } else {
    Csr csr;
    csr_from_triplets((size_t)n_ind, ff, csr);
    std::vector<Trip>().swap(ff);
    const double t3 = now_s();
    info[1] = (double)csr.data.size();
    std::vector<double> x(n_ind, 0.0);
    double bn = 0.0;
    for (double v : rhs) bn += v * v;
    info[10] = std::sqrt(bn);
    int st = OK;
    if (solver == 1) {
      if ((double)n_ind * (double)n_ind > 4.0e8) return ERR_INVALID_ARG;
      std::vector<double> dense((size_t)n_ind * n_ind, 0.0);
      for (int64_t i = 0; i < n_ind; ++i)
        for (uint64_t k = csr.indptr[i]; k < csr.indptr[i + 1]; ++k)
          dense[(size_t)i * n_ind + csr.indices[k]] = csr.data[k];
      st = chol_solve(dense.data(), (size_t)n_ind, rhs.data(), x.data());
      info[2] = 1;
      info[3] = st == OK ? residual_of(csr, x.data(), rhs.data()) : 0.0;
    } else {
      size_t mi = max_iter > 0 ? (size_t)max_iter : std::max<size_t>(4 * (size_t)n_ind, 200);
      size_t iters = 0;
      double res = 0.0;
      st = pcg(csr, rhs.data(), tol, mi, nthreads, x.data(), &iters, &res);
      info[2] = (double)iters;
      info[3] = res;
    }
    const double t4 = now_s();
    info[6] = t3 - t2;
    info[7] = t4 - t3;
    if (st) return st;
    for (int64_t d = 0; d < ndof; ++d) u[d] = u0[d] + (ind_of[d] >= 0 ? 1.0 * x[ind_of[d]] : 0.0);
    if (csr_out) {
      OrCsr* h = new OrCsr;
      h->csr = std::move(csr);
      *csr_out = h;
    }
    if (rhs_out) std::copy(rhs.begin(), rhs.end(), rhs_out);
  }
  for (int64_t d = 0; d < ndof; ++d) u_full[d] = u[d];
  if (rf_full) {  // analysis.rs:1027-1035
    std::vector<double> ku(ndof, 0.0);
    for (const Trip& t : trips) ku[t.i] += t.v * u[t.j];
    for (int64_t d = 0; d < ndof; ++d) rf_full[d] = ku[d] - f_full[d];
  }
  info[4] = t1 - t0;
  info[5] = t2 - t1;
  info[8] = now_s() - t0;
  return OK;
}

int64_t or_csr_n(const OrCsr* h) { return (int64_t)h->csr.n; }
int64_t or_csr_nnz(const OrCsr* h) { return (int64_t)h->csr.data.size(); }
void or_csr_export(const OrCsr* h, int64_t* indptr, int64_t* indices, double* data) {
  for (size_t i = 0; i <= h->csr.n; ++i) indptr[i] = (int64_t)h->csr.indptr[i];
  for (size_t k = 0; k < h->csr.data.size(); ++k) {
    indices[k] = (int64_t)h->csr.indices[k];
    data[k] = h->csr.data[k];
  }
}
void or_csr_free(OrCsr* h) { delete h; }

// ---------------------------------------------------------------------------
// DofMap with multi-point constraints (constraint.rs:8-136, 138-172, 207-217,
// coalesce 219-235).  An MPC is u_slave = sum_m alpha_m u_m + u0.  Prescribed
// DOFs: later entries of the list win (the HashMap insert of analysis.rs:556-565).
// ---------------------------------------------------------------------------
struct OrDofMap {
  int64_t n_full = 0, n_ind = 0;
  std::vector<double> u0;
  std::vector<std::vector<std::pair<int64_t, double>>> t_row;
  std::vector<int64_t> ind_of;
};

namespace {
// constraint.rs:219-235: stable sort by DOF, merge equal DOFs in order, a run
// starts only with a non-zero term, then drop |alpha| <= 1e-16
std::vector<std::pair<int64_t, double>> coalesce(std::vector<std::pair<int64_t, double>> terms) {
  std::stable_sort(terms.begin(), terms.end(),
                   [](const std::pair<int64_t, double>& a, const std::pair<int64_t, double>& b) { return a.first < b.first; });
  std::vector<std::pair<int64_t, double>> out;
  for (const auto& t : terms) {
    if (!out.empty() && out.back().first == t.first) {
      out.back().second += t.second;
      continue;
    }
    if (std::fabs(t.second) > 0.0) out.push_back(t);
  }
  std::vector<std::pair<int64_t, double>> kept;
  for (const auto& t : out)
    if (std::fabs(t.second) > 1e-16) kept.push_back(t);
  return kept;
}
}  // namespace

// mpc_ptr [n_mpc+1] delimits each MPC's masters in mpc_master / mpc_alpha.
int or_dofmap_build(int64_t ndof, int64_t n_presc, const int64_t* presc_dof, const double* presc_val, int64_t n_mpc,
                    const int64_t* mpc_slave, const int64_t* mpc_ptr, const int64_t* mpc_master,
                    const double* mpc_alpha, const double* mpc_u0, OrDofMap** out) {
  auto* m = new OrDofMap();
  m->n_full = ndof;
  m->u0.assign(ndof, 0.0);
  std::vector<char> is_presc(ndof, 0);
  std::vector<double> presc(ndof, 0.0);
  for (int64_t k = 0; k < n_presc; ++k) {
    const int64_t d = presc_dof[k];
    if (d < 0 || d >= ndof) continue;
    is_presc[d] = 1;
    presc[d] = presc_val[k];
  }
  for (int64_t d = 0; d < ndof; ++d)
    if (is_presc[d]) m->u0[d] = presc[d];
  // slave_of: the last MPC naming a slave wins (HashMap::insert replaces)
  std::vector<int64_t> slave_of(ndof, -1);
  for (int64_t i = 0; i < n_mpc; ++i) {
    const int64_t s = mpc_slave[i];
    if (s < 0 || s >= ndof) continue;
    if (is_presc[s]) continue;
    slave_of[s] = i;
  }
  std::vector<std::vector<std::pair<int64_t, double>>> alphas(ndof);
  for (int64_t si = 0; si < n_mpc; ++si) {
    const int64_t s = mpc_slave[si];
    if (s < 0 || s >= ndof || slave_of[s] != si) continue;
    std::vector<std::pair<int64_t, double>> terms;
    for (int64_t k = mpc_ptr[si]; k < mpc_ptr[si + 1]; ++k) terms.push_back({mpc_master[k], mpc_alpha[k]});
    double particular = mpc_u0[si];
    for (int pass = 0; pass < 32; ++pass) {
      std::vector<std::pair<int64_t, double>> next;
      bool changed = false;
      for (const auto& t : terms) {
        const int64_t d = t.first;
        const double a = t.second;
        const int64_t k = (d >= 0 && d < ndof) ? slave_of[d] : -1;
        if (k >= 0) {
          changed = true;
          particular += a * mpc_u0[k];
          for (int64_t q = mpc_ptr[k]; q < mpc_ptr[k + 1]; ++q) next.push_back({mpc_master[q], a * mpc_alpha[q]});
        } else {
          next.push_back({d, a});
        }
      }
      terms = coalesce(next);
      if (!changed) break;
    }
    std::vector<std::pair<int64_t, double>> ind_terms;
    for (const auto& t : terms) {
      const int64_t d = t.first;
      if (d < 0 || d >= ndof) {
        delete m;
        return ERR_INVALID_ARG;
      }
      if (is_presc[d]) {
        particular += t.second * presc[d];
      } else if (slave_of[d] >= 0) {
        delete m;
        return ERR_INVALID_ARG;  // "MPC: zyklische Mehrpunktbedingung."
      } else {
        ind_terms.push_back(t);
      }
    }
    alphas[s] = ind_terms;
    m->u0[s] = particular;
  }
  std::vector<char> is_ind(ndof, 1);
  bool any_slave = false;
  for (int64_t d = 0; d < ndof; ++d) {
    if (is_presc[d]) is_ind[d] = 0;
    if (slave_of[d] >= 0) {
      is_ind[d] = 0;
      any_slave = true;
    }
  }
  m->ind_of.assign(ndof, -1);
  for (int64_t d = 0; d < ndof; ++d)
    if (is_ind[d]) m->ind_of[d] = m->n_ind++;
  bool any_presc = false;
  for (int64_t d = 0; d < ndof; ++d) any_presc = any_presc || is_presc[d];
  if (m->n_ind == 0 && !any_slave && !any_presc) {
    delete m;
    return ERR_NO_FREE_DOF;
  }
  m->t_row.assign(ndof, {});
  for (int64_t d = 0; d < ndof; ++d) {
    if (is_ind[d]) {
      m->t_row[d].push_back({m->ind_of[d], 1.0});
    } else if (slave_of[d] >= 0) {
      for (const auto& t : alphas[d]) {
        const int64_t col = m->ind_of[t.first];
        if (col >= 0 && std::fabs(t.second) > 0.0) m->t_row[d].push_back({col, t.second});
      }
    }
  }
  *out = m;
  return OK;
}

int64_t or_dofmap_n_ind(const OrDofMap* m) { return m->n_ind; }

// T as CSR over full DOFs (t_ptr [n_full+1], t_col, t_val) and u0
int64_t or_dofmap_export(const OrDofMap* m, int64_t* t_ptr, int64_t* t_col, double* t_val, double* u0) {
  int64_t k = 0;
  for (int64_t d = 0; d < m->n_full; ++d) {
    if (t_ptr) t_ptr[d] = k;
    for (const auto& t : m->t_row[d]) {
      if (t_col) t_col[k] = t.first;
      if (t_val) t_val[k] = t.second;
      ++k;
    }
  }
  if (t_ptr) t_ptr[m->n_full] = k;
  if (u0)
    for (int64_t d = 0; d < m->n_full; ++d) u0[d] = m->u0[d];
  return k;
}

void or_dofmap_free(OrDofMap* m) { delete m; }

// DofMap::reduce (constraint.rs:138-172) followed by csr_from_triplets and the
// chosen solver, then reconstruct (207-217): the MPC path of solve_linear
// (analysis.rs:1018-1025).  CSR of K_ff and rhs returned through the handle.
int or_solve_reduced(const OrDofMap* m, int64_t nt, const int64_t* ti, const int64_t* tj, const double* tv,
                     const double* f_full, int solver, double tol, int64_t max_iter, double* u_full, double* info,
                     OrCsr** csr_out, double* rhs_out) {
  const int64_t n = m->n_ind;
  std::vector<double> rhs(n, 0.0);
  for (int64_t i = 0; i < m->n_full; ++i) {
    const double fi = f_full[i];
    if (std::fabs(fi) == 0.0) continue;
    for (const auto& t : m->t_row[i]) rhs[t.first] += t.second * fi;
  }
  std::vector<Trip> ff;
  for (int64_t k = 0; k < nt; ++k) {
    const int64_t i = ti[k], j = tj[k];
    const double v = tv[k];
    if (i < 0 || j < 0 || i >= m->n_full || j >= m->n_full || std::fabs(v) == 0.0) continue;
    const double u0j = m->u0[j];
    for (const auto& a : m->t_row[i]) {
      if (std::fabs(u0j) > 0.0) rhs[a.first] -= v * a.second * u0j;
      for (const auto& b : m->t_row[j]) ff.push_back({(uint64_t)a.first, (uint64_t)b.first, v * a.second * b.second});
    }
  }
  auto* h = new OrCsr();
  csr_from_triplets((size_t)n, ff, h->csr);
  std::vector<double> x(n, 0.0);
  int st = OK;
  if (solver == 1) {
    std::vector<double> dense((size_t)n * n, 0.0);
    for (int64_t i = 0; i < n; ++i)
      for (uint64_t k = h->csr.indptr[i]; k < h->csr.indptr[i + 1]; ++k)
        dense[(size_t)i * n + h->csr.indices[k]] = h->csr.data[k];
    st = chol_solve(dense.data(), (size_t)n, rhs.data(), x.data());
    info[0] = 1;
    info[1] = st == OK ? residual_of(h->csr, x.data(), rhs.data()) : 0.0;
  } else {
    size_t mi = max_iter > 0 ? (size_t)max_iter : std::max<size_t>(4 * (size_t)n, 200);
    size_t iters = 0;
    double res = 0.0;
    st = pcg(h->csr, rhs.data(), tol, mi, 1, x.data(), &iters, &res);
    info[0] = (double)iters;
    info[1] = res;
  }
  for (int64_t d = 0; d < m->n_full; ++d) {
    double u = m->u0[d];
    for (const auto& t : m->t_row[d]) u += t.second * x[t.first];
    u_full[d] = u;
  }
  if (rhs_out)
    for (int64_t i = 0; i < n; ++i) rhs_out[i] = rhs[i];
  if (csr_out)
    *csr_out = h;
  else
    delete h;
  return st;
}

// solve_kff's CSR + backend part (linalg.rs:311-404) on caller triplets:
// csr_from_triplets, then dense Cholesky (solver=1) or PCG (solver=2).
// info = {iters, residual}.
int or_solve_kff(int64_t n, int64_t nt, const int64_t* ti, const int64_t* tj, const double* tv,
                 const double* rhs, int solver, double tol, int64_t max_iter, int nthreads, double* x,
                 double* info) {
  std::vector<Trip> trips(nt);
  for (int64_t k = 0; k < nt; ++k) trips[k] = {(uint64_t)ti[k], (uint64_t)tj[k], tv[k]};
  Csr csr;
  csr_from_triplets((size_t)n, trips, csr);
  if (solver == 1) {
    std::vector<double> dense((size_t)n * n, 0.0);
    for (int64_t i = 0; i < n; ++i)
      for (uint64_t k = csr.indptr[i]; k < csr.indptr[i + 1]; ++k)
        dense[(size_t)i * n + csr.indices[k]] = csr.data[k];
    int st = chol_solve(dense.data(), (size_t)n, rhs, x);
    info[0] = 1;
    info[1] = st == OK ? residual_of(csr, x, rhs) : 0.0;
    return st;
  }
  size_t mi = max_iter > 0 ? (size_t)max_iter : std::max<size_t>(4 * (size_t)n, 200);
  size_t iters = 0;
  double res = 0.0;
  int st = pcg(csr, rhs, tol, mi, nthreads, x, &iters, &res);
  info[0] = (double)iters;
  info[1] = res;
  return st;
}

// Nodal averaged stresses (analysis.rs:1061-1153 without thermal terms):
// element nodal stresses (hex8_nodal_stress / hex20_nodal_stress), summed per
// node in element order and divided by the number of contributing elements;
// von Mises per node (elem.rs:651-660).  stress [n_nodes][6], vm [n_nodes],
// emean [n_elem][6] = mean of the element's nodal stresses ("stress_gp",
// analysis.rs:1141-1152); vm and emean may be null.
int or_nodal_stress(int64_t n_nodes, const double* coords, int nn, int reduced, int64_t n_elem, const int32_t* conn,
                    const double* e_elem, double nu, const double* u_full, double* stress, double* vm, double* emean,
                    int64_t* bad) {
  std::vector<double> acc((size_t)n_nodes * 6, 0.0), cnt(n_nodes, 0.0);
  double xyz[60], ue[60], sn[20][6];
  for (int64_t e = 0; e < n_elem; ++e) {
    const int32_t* c = conn + e * nn;
    for (int a = 0; a < nn; ++a)
      for (int q = 0; q < 3; ++q) {
        xyz[3 * a + q] = coords[3 * (int64_t)c[a] + q];
        ue[3 * a + q] = u_full[3 * (int64_t)c[a] + q];
      }
    int st = (nn == 8 && reduced == 1) ? hex8r_nodal_stress(xyz, ue, e_elem[e], nu, sn)
             : nn == 8  ? hex8_nodal_stress(xyz, ue, e_elem[e], nu, sn)
             : nn == 20 ? hex20_nodal_stress(xyz, ue, e_elem[e], nu, reduced != 0, sn)
             : nn == 10 ? tet10_nodal_stress(xyz, ue, e_elem[e], nu, sn)
             : nn == 6  ? wedge_nodal_stress<6>(xyz, ue, e_elem[e], nu, sn)
             : nn == 15 ? wedge_nodal_stress<15>(xyz, ue, e_elem[e], nu, sn)
                        : tet4_nodal_stress(xyz, ue, e_elem[e], nu, sn);
    if (st) {
      *bad = e;
      return st;
    }
    for (int a = 0; a < nn; ++a) {
      for (int k = 0; k < 6; ++k) acc[6 * (size_t)c[a] + k] += sn[a][k];
      cnt[c[a]] += 1.0;
    }
    if (emean)
      for (int k = 0; k < 6; ++k) {
        double m = 0.0;
        for (int a = 0; a < nn; ++a) m += sn[a][k] / (double)nn;
        emean[6 * e + k] = m;
      }
  }
  for (int64_t i = 0; i < n_nodes; ++i) {
    for (int k = 0; k < 6; ++k) stress[6 * i + k] = cnt[i] > 0.0 ? acc[6 * i + k] / cnt[i] : 0.0;
    if (vm) vm[i] = von_mises(stress + 6 * i);
  }
  return OK;
}

// Reactions K u - f over the raw element triplets (analysis.rs:1027-1035).
int or_reactions(int64_t n_nodes, const double* coords, int nn, int reduced, int64_t n_elem, const int32_t* conn,
                 const double* e_elem, double nu, const double* u_full, const double* f_full, double* rf,
                 int64_t* bad) {
  const int m = 3 * nn;
  std::vector<double> ke((size_t)m * m), ku(3 * (size_t)n_nodes, 0.0);
  double xyz[60], vol;
  for (int64_t e = 0; e < n_elem; ++e) {
    const int32_t* c = conn + e * nn;
    for (int a = 0; a < nn; ++a)
      for (int q = 0; q < 3; ++q) xyz[3 * a + q] = coords[3 * (int64_t)c[a] + q];
    int st = element_ke(nn, xyz, e_elem[e], nu, reduced, ke.data(), &vol);
    if (st) {
      *bad = e;
      return st;
    }
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) {
        const double v = ke[(size_t)i * m + j];
        if (std::fabs(v) > 0.0)
          ku[3 * (size_t)c[i / 3] + i % 3] += v * u_full[3 * (size_t)c[j / 3] + j % 3];
      }
  }
  for (int64_t d = 0; d < 3 * n_nodes; ++d) rf[d] = ku[d] - f_full[d];
  return OK;
}

// K u_k - f_k for nvec vectors at once (u, f, rf: [nvec][3 n_nodes]) with the
// element stiffness of the restated element_ke, the reactions of
// analysis.rs:1027-1035 without triplets: element by element, Ke computed once
// per element and applied to every vector.  nthreads > 1 splits the element
// loop into nthreads contiguous ranges with their own accumulators, added in
// range order (the result depends on nthreads only through that order).
// Used as a residual check of solutions computed elsewhere: no K is stored,
// so it reaches meshes whose triplet lists would not fit in host memory.
int or_residual_multi(int64_t n_nodes, const double* coords, int nn, int reduced, int64_t n_elem,
                      const int32_t* conn, const double* e_elem, double nu, int64_t nvec, const double* u,
                      const double* f, double* rf, int nthreads, int64_t* bad) {
  const int m = 3 * nn;
  const int64_t ndof = 3 * n_nodes;
  if (nthreads < 1) nthreads = 1;
  std::vector<std::vector<double>> acc(nthreads);
  std::vector<int64_t> first_bad(nthreads, -1);
  std::vector<int> first_st(nthreads, OK);
#pragma omp parallel num_threads(nthreads)
  {
    const int t = omp_get_thread_num(), nt = omp_get_num_threads();
    const int64_t e0 = n_elem * t / nt, e1 = n_elem * (t + 1) / nt;
    std::vector<double>& ku = acc[t];
    ku.assign((size_t)nvec * ndof, 0.0);
    std::vector<double> ke((size_t)m * m);
    double xyz[60], vol;
    for (int64_t e = e0; e < e1; ++e) {
      const int32_t* c = conn + e * nn;
      for (int a = 0; a < nn; ++a)
        for (int q = 0; q < 3; ++q) xyz[3 * a + q] = coords[3 * (int64_t)c[a] + q];
      const int st = element_ke(nn, xyz, e_elem[e], nu, reduced, ke.data(), &vol);
      if (st) {
        first_bad[t] = e;
        first_st[t] = st;
        break;
      }
      for (int64_t k = 0; k < nvec; ++k) {
        const double* uk = u + k * ndof;
        double* yk = ku.data() + k * ndof;
        for (int i = 0; i < m; ++i) {
          double s = 0.0;
          for (int j = 0; j < m; ++j) s += ke[(size_t)i * m + j] * uk[3 * (int64_t)c[j / 3] + j % 3];
          yk[3 * (int64_t)c[i / 3] + i % 3] += s;
        }
      }
    }
  }
  for (int t = 0; t < nthreads; ++t)
    if (first_st[t]) {
      *bad = first_bad[t];
      return first_st[t];
    }
  const int64_t tot = nvec * ndof;
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (int64_t d = 0; d < tot; ++d) {
    double s = 0.0;
    for (int t = 0; t < nthreads; ++t)
      if (!acc[t].empty()) s += acc[t][d];
    rf[d] = s - f[d];
  }
  return OK;
}

// ||K x - b|| <= 1e-8 max(||b||, 1) + 1e-10 (sparse_native.rs:1572-1578)
int or_residual_ok(double residual, double bnorm) {
  return std::isfinite(residual) && residual <= 1e-8 * std::max(bnorm, 1.0) + 1e-10;
}

// Compliance gradient, no reference counterpart: for every element,
// g_e = -p rho_e^(p-1) E0 u_e^T K_e(E=1, nu) u_e with K_e from the restated
// hex8 / hex20 stiffness.  Returns the first failing element in *bad.
int or_compliance_grad(int64_t n_nodes, const double* coords, int nn, int reduced, int64_t n_elem,
                       const int32_t* conn, const double* rho, double pexp, double e0, double nu,
                       const double* u_full, double* grad, int64_t* bad) {
  const int m = 3 * nn;
  std::vector<double> ke((size_t)m * m);
  double xyz[60], ue[60], vol;
  for (int64_t e = 0; e < n_elem; ++e) {
    const int32_t* c = conn + e * nn;
    for (int a = 0; a < nn; ++a)
      for (int q = 0; q < 3; ++q) {
        xyz[3 * a + q] = coords[3 * (int64_t)c[a] + q];
        ue[3 * a + q] = u_full[3 * (int64_t)c[a] + q];
      }
    int st = element_ke(nn, xyz, 1.0, nu, reduced, ke.data(), &vol);
    if (st) {
      *bad = e;
      return st;
    }
    double s = 0.0;
    for (int i = 0; i < m; ++i) {
      double row = 0.0;
      for (int j = 0; j < m; ++j) row += ke[(size_t)i * m + j] * ue[j];
      s += ue[i] * row;
    }
    grad[e] = -pexp * std::pow(rho[e], pexp - 1.0) * e0 * s;
  }
  (void)n_nodes;
  return OK;
}

}  // extern "C"
