// recover.cu -- nodal stress recovery and reactions after a solve.
//
// Replaces, for C3D8 / C3D8R / C3D8I / C3D20 / C3D20R / C3D4 / C3D10 / C3D6 / C3D15
// with an isotropic material, the post-solve loops of the reference's solve_linear:
//   reactions      solver/src/analysis.rs:1027-1035   ku = sum of element K u, rf = ku - f
//   nodal stresses solver/src/analysis.rs:1061-1153   element nodal stresses summed per
//                                                     node in element order / element count
//   strain, vm     solver/src/analysis.rs:1154-1174, von_mises elem.rs:651-660
//   element stress hex8_nodal_stress elem.rs:744-779 (Gauss points HEX_XI*G2, extrapolated
//                  with the trilinear shapes at HEX_XI*sqrt(3)); hex20_nodal_stress and
//                  hex20_extrapolate quadratic.rs:148-225 (hex_gauss points, tensor-product
//                  Lagrange extrapolation, lagrange1d quadratic.rs:227-244)
//                  tet4_nodal_stress elem.rs:781-795 (one constant stress), tet10_nodal_stress
//                  quadratic.rs:678-702 (stress evaluated at the ten nodes);
//                  wedge6_nodal_stress / wedge15_nodal_stress extra.rs:134-153, 821-850
//                  (stress evaluated at the nodes)
//   element mean   "stress_gp" analysis.rs:1141-1152 (mean of the element's nodal stresses)
//
// Two kernels.  element_recover_kernel: lanes are (element, Gauss point)
// pairs, as in the energy kernel; each lane forms J, its cofactors and the
// displacement gradient, and the stress sigma = D eps (d_iso_3d of the
// element's E).  After a warp sync, lanes become (element, node) pairs: each
// extrapolates the node's stress from the element's Gauss-point stresses and
// integrates the node's internal force f_a = sum_g w det J B_a^T sigma_g,
// which is row a of K_e u_e.  It writes 9 numbers per (element, node).
// k_recover_nodes: one thread per node walks the node's incident elements in
// ascending order (the reference's element loop order) and averages the
// stresses, sums the forces, and writes stress, strain, von Mises and
// rf = K u - f.
#include <algorithm>
#include <cmath>
#include <vector>

#include "solver.cuh"

int element_tables_for(axia_ctx* ctx, int nn, int ng, const double** dn, const double** w);
void element_dshape(int nn, double r, double s, double t, double* dn);

namespace {

const double kG2 = 0.5773502691896257;
const double kG3[3] = {-0.7745966692414834, 0.0, 0.7745966692414834};
const int kXi[20][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1}, {-1, -1, 1},
                        {1, -1, 1},   {1, 1, 1},   {-1, 1, 1}, {0, -1, -1}, {1, 0, -1},
                        {0, 1, -1},   {-1, 0, -1}, {0, -1, 1}, {1, 0, 1},   {0, 1, 1},
                        {-1, 0, 1},   {-1, -1, 0}, {1, -1, 0}, {1, 1, 0},   {-1, 1, 0}};

constexpr int kRec = 9;  // per (element, node): 6 stresses, 3 forces
constexpr int kGp = 15;  // per Gauss point in shared memory: w*cofactor (9), sigma (6)

template <int NN, int NG>
struct RecoverCfg {
  static constexpr int EPW = 32 / NG;           // elements per warp step
  static constexpr int WARPS = NN == 8 ? 8 : 4;
  static constexpr int ND = 3 * NN;
};

template <int NN, int NG>
__global__ void __launch_bounds__(32 * RecoverCfg<NN, NG>::WARPS)
element_recover_kernel(int64_t n_elem, const int32_t* __restrict__ conn, const double* __restrict__ coords,
                       const double* __restrict__ u, const double* __restrict__ e_elem, double nu,
                       const double* __restrict__ dn_tab, const double* __restrict__ w_tab,
                       const double* __restrict__ x_tab, const int* __restrict__ perm, double* __restrict__ rec,
                       double* __restrict__ emean, DevStatus* st) {
  using C = RecoverCfg<NN, NG>;
  constexpr int EPW = C::EPW, WARPS = C::WARPS, ND = C::ND;
  __shared__ double s_dn[NG * NN * 3];
  __shared__ double s_w[NG];
  __shared__ double s_x[NN * NG];
  __shared__ int s_perm[NG];
  // per warp: coordinates and displacements of its elements, later the nodal stresses
  __shared__ double s_a[WARPS][2 * EPW * ND];
  __shared__ double s_gp[WARPS][EPW * NG * kGp];
  for (int t = threadIdx.x; t < NG * NN * 3; t += blockDim.x) s_dn[t] = dn_tab[t];
  for (int t = threadIdx.x; t < NN * NG; t += blockDim.x) s_x[t] = x_tab[t];
  for (int t = threadIdx.x; t < NG; t += blockDim.x) {
    s_w[t] = w_tab[t];
    s_perm[t] = perm[t];
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int le = lane / NG, g = lane % NG;
  double* A = s_a[warp];
  double* GP = s_gp[warp];
  const int64_t step = (int64_t)gridDim.x * WARPS * EPW;
  const double onu = 1.0 + nu;
  for (int64_t e0 = ((int64_t)blockIdx.x * WARPS + warp) * EPW; e0 < n_elem; e0 += step) {
    for (int t = lane; t < EPW * ND; t += 32) {
      const int k = t / ND, c = t % ND;
      const int64_t e = e0 + k;
      double xv = 0.0, uv = 0.0;
      if (e < n_elem) {
        const int64_t node = conn[e * NN + c / 3];
        xv = coords[3 * node + c % 3];
        uv = u[3 * node + c % 3];
      }
      A[t] = xv;
      A[EPW * ND + t] = uv;
    }
    __syncwarp();
    {
      const int64_t e = e0 + le;
      if (le < EPW && e < n_elem) {
        const double* X = A + le * ND;
        const double* U = A + EPW * ND + le * ND;
        const double* dn = s_dn + g * NN * 3;
        double J[3][3] = {}, Gu[3][3] = {};
#pragma unroll 4
        for (int a = 0; a < NN; ++a) {
          const double d0 = dn[3 * a], d1 = dn[3 * a + 1], d2 = dn[3 * a + 2];
#pragma unroll
          for (int q = 0; q < 3; ++q) {
            const double xq = X[3 * a + q], uq = U[3 * a + q];
            J[q][0] = fma(d0, xq, J[q][0]);
            J[q][1] = fma(d1, xq, J[q][1]);
            J[q][2] = fma(d2, xq, J[q][2]);
            Gu[0][q] = fma(d0, uq, Gu[0][q]);
            Gu[1][q] = fma(d1, uq, Gu[1][q]);
            Gu[2][q] = fma(d2, uq, Gu[2][q]);
          }
        }
        // cofactors: inverse Jacobian = b / det (invert3 elem.rs:10-29)
        double b[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            const int j1 = (j + 1) % 3, j2 = (j + 2) % 3, i1 = (i + 1) % 3, i2 = (i + 2) % 3;
            b[i][j] = J[j1][i1] * J[j2][i2] - J[j1][i2] * J[j2][i1];
          }
        double det = J[0][0] * b[0][0] + J[0][1] * b[1][0] + J[0][2] * b[2][0];
        if (!(fabs(det) >= 1e-18)) {
          record_error(st, e, isfinite(det) ? AXIA_ERR_SINGULAR_JACOBIAN : AXIA_ERR_NONFINITE);
          det = 1.0;
        } else if (det <= 0.0 && s_w[g] > 0.0) {  // integration points only
          record_error(st, e, AXIA_ERR_NEG_JACOBIAN);
        }
        const double E = e_elem[e];
        if (!(E > 0.0)) record_error(st, e, AXIA_ERR_MATERIAL);
        const double lam = E * nu / (onu * (1.0 - 2.0 * nu));
        const double mu = E / (2.0 * onu);
        const double inv = 1.0 / det;
        // du_q/dx_i = sum_p b[p][i] Gu[p][q] / det
        double H[3][3];
#pragma unroll
        for (int q = 0; q < 3; ++q)
#pragma unroll
          for (int i = 0; i < 3; ++i)
            H[q][i] = fma(b[0][i], Gu[0][q], fma(b[1][i], Gu[1][q], b[2][i] * Gu[2][q])) * inv;
        // Voigt xx yy zz xy yz zx, engineering shears (fill_b3 elem.rs:114-132)
        const double exx = H[0][0], eyy = H[1][1], ezz = H[2][2];
        const double gxy = H[0][1] + H[1][0], gyz = H[1][2] + H[2][1], gzx = H[2][0] + H[0][2];
        double* P = GP + (le * NG + g) * kGp;
        const double wg = s_w[g];
#pragma unroll
        for (int p = 0; p < 3; ++p)
#pragma unroll
          for (int i = 0; i < 3; ++i) P[3 * p + i] = wg * b[p][i];
        const double l2m = lam + 2.0 * mu;
        P[9] = l2m * exx + lam * eyy + lam * ezz;
        P[10] = lam * exx + l2m * eyy + lam * ezz;
        P[11] = lam * exx + lam * eyy + l2m * ezz;
        P[12] = mu * gxy;
        P[13] = mu * gyz;
        P[14] = mu * gzx;
      }
    }
    __syncwarp();
    // (element, node) tasks; A now holds the nodal stresses
    for (int t = lane; t < EPW * NN; t += 32) {
      const int k = t / NN, a = t % NN;
      const int64_t e = e0 + k;
      if (e >= n_elem) continue;
      double s[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, f0 = 0.0, f1 = 0.0, f2 = 0.0;
      const double* xrow = s_x + a * NG;
#pragma unroll 4
      for (int m = 0; m < NG; ++m) {
        const int gg = s_perm[m];
        const double* P = GP + (k * NG + gg) * kGp;
        const double* dn = s_dn + (gg * NN + a) * 3;
        // w det dN_a/dx_i = w sum_p b[p][i] dN_a/dxi_p
        const double gx = P[0] * dn[0] + P[3] * dn[1] + P[6] * dn[2];
        const double gy = P[1] * dn[0] + P[4] * dn[1] + P[7] * dn[2];
        const double gz = P[2] * dn[0] + P[5] * dn[1] + P[8] * dn[2];
        f0 += gx * P[9] + gy * P[12] + gz * P[14];
        f1 += gy * P[10] + gx * P[12] + gz * P[13];
        f2 += gz * P[11] + gy * P[13] + gx * P[14];
        const double xw = xrow[m];
#pragma unroll
        for (int c = 0; c < 6; ++c) s[c] += xw * P[9 + c];
      }
      double* out = rec + (e * NN + a) * kRec;
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        out[c] = s[c];
        A[(k * NN + a) * 6 + c] = s[c];
      }
      out[6] = f0;
      out[7] = f1;
      out[8] = f2;
    }
    if (emean) {
      __syncwarp();
      for (int t = lane; t < EPW * 6; t += 32) {
        const int k = t / 6, c = t % 6;
        const int64_t e = e0 + k;
        if (e >= n_elem) continue;
        double m = 0.0;
        for (int a = 0; a < NN; ++a) m += A[(k * NN + a) * 6 + c] / (double)NN;
        emean[e * 6 + c] = m;
      }
    }
    __syncwarp();
  }
}

// One thread per node: average over the incident elements in ascending order.
__global__ void k_recover_nodes(int64_t n_nodes, int nn, const int64_t* __restrict__ ne_ptr,
                                const int32_t* __restrict__ ne, const double* __restrict__ rec,
                                const double* __restrict__ f, double nu, double e_strain, double* __restrict__ stress,
                                double* __restrict__ strain, double* __restrict__ vm, double* __restrict__ rf) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_nodes;
       i += (int64_t)gridDim.x * blockDim.x) {
    double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, ku[3] = {0.0, 0.0, 0.0}, cnt = 0.0;
    for (int64_t k = ne_ptr[i]; k < ne_ptr[i + 1]; ++k) {
      const int32_t packed = ne[k];
      const int64_t e = packed >> 5;
      const int a = packed & 31;
      const double* r = rec + (e * nn + a) * kRec;
#pragma unroll
      for (int c = 0; c < 6; ++c) acc[c] += r[c];
      ku[0] += r[6];
      ku[1] += r[7];
      ku[2] += r[8];
      cnt += 1.0;
    }
    double s[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) s[c] = cnt > 0.0 ? acc[c] / cnt : 0.0;
    if (stress) {
#pragma unroll
      for (int c = 0; c < 6; ++c) stress[6 * i + c] = s[c];
    }
    if (vm) {
      const double dxy = s[0] - s[1], dyz = s[1] - s[2], dzx = s[2] - s[0];
      vm[i] = sqrt(0.5 * (dxy * dxy + dyz * dyz + dzx * dzx) + 3.0 * (s[3] * s[3] + s[4] * s[4] + s[5] * s[5]));
    }
    if (strain) {
      const double tr = s[0] + s[1] + s[2];
      const double g2 = e_strain / (1.0 + nu);
#pragma unroll
      for (int c = 0; c < 3; ++c) strain[6 * i + c] = ((1.0 + nu) * s[c] - nu * tr) / e_strain;
#pragma unroll
      for (int c = 3; c < 6; ++c) strain[6 * i + c] = s[c] / g2;
    }
    if (rf) {
#pragma unroll
      for (int q = 0; q < 3; ++q) rf[3 * i + q] = ku[q] - (f ? f[3 * i + q] : 0.0);
    }
  }
}

// one warp per C3D8 element: rows 0..23 of K_e u_e into the force slots of rec
__global__ void k_ke_force(int64_t n_elem, const int32_t* __restrict__ conn, const double* __restrict__ ke,
                           const double* __restrict__ u, double* __restrict__ rec) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t e = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); e < n_elem; e += warps) {
    const double ue = lane < 24 ? u[3 * (int64_t)conn[e * 8 + lane / 3] + lane % 3] : 0.0;
    double f = 0.0;
    const double* row = ke + e * 576 + (int64_t)(lane < 24 ? lane : 0) * 24;
    for (int j = 0; j < 24; ++j) {
      const double uj = __shfl_sync(0xffffffffu, ue, j);
      f = fma(row[j], uj, f);
    }
    if (lane < 24) rec[(e * 8 + lane / 3) * kRec + 6 + lane % 3] = f;
  }
}

// lagrange1d quadratic.rs:227-244
void lagrange_weights(const double* pts, int n, double x, double* w) {
  for (int i = 0; i < n; ++i) {
    w[i] = 1.0;
    for (int j = 0; j < n; ++j)
      if (i != j) w[i] *= (x - pts[j]) / (pts[i] - pts[j]);
  }
}

// Extrapolation matrix X[a][m] (node a, m-th Gauss point of the reference's
// order) and perm[m] = index of that point in the element tables.
void extrapolation_table(int nn, int ng, std::vector<double>& x, std::vector<int>& perm) {
  x.assign((size_t)nn * ng, 0.0);
  perm.resize(ng);
  if (nn == 8) {
    // reference order HEX_XI[m] * G2; the tables run xi, eta, zeta from - to +
    const double s3 = std::sqrt(3.0);
    for (int m = 0; m < 8; ++m)
      perm[m] = 4 * (kXi[m][0] > 0) + 2 * (kXi[m][1] > 0) + (kXi[m][2] > 0);
    for (int a = 0; a < 8; ++a) {
      const double xi = kXi[a][0] * s3, eta = kXi[a][1] * s3, zeta = kXi[a][2] * s3;
      for (int m = 0; m < 8; ++m)
        x[(size_t)a * 8 + m] = 0.125 * (1.0 + kXi[m][0] * xi) * (1.0 + kXi[m][1] * eta) * (1.0 + kXi[m][2] * zeta);
    }
    return;
  }
  const double p2[2] = {-kG2, kG2};
  const double* pts = ng == 8 ? p2 : kG3;
  const int n1 = ng == 8 ? 2 : 3;
  for (int m = 0; m < ng; ++m) perm[m] = m;
  for (int a = 0; a < 20; ++a) {
    double lx[3], ly[3], lz[3];
    lagrange_weights(pts, n1, kXi[a][0], lx);
    lagrange_weights(pts, n1, kXi[a][1], ly);
    lagrange_weights(pts, n1, kXi[a][2], lz);
    int m = 0;
    for (int i = 0; i < n1; ++i)
      for (int j = 0; j < n1; ++j)
        for (int k = 0; k < n1; ++k, ++m) x[(size_t)a * ng + m] = lx[i] * ly[j] * lz[k];
  }
}

struct XTab {
  double* x = nullptr;
  int* perm = nullptr;
  int device = -1;
};
XTab g_xtab[8];  // hex8, hex20, hex20r, tet4, tet10, hex8r, wedge6, wedge15

// The points the recovery kernel evaluates and how nodes take their stress:
//  * hexahedra: the stiffness Gauss points, extrapolated to the nodes (X above);
//  * C3D4: its one point (constant stress, elem.rs:781-795), every node takes it;
//  * C3D10, C3D6, C3D15: the stiffness Gauss points (for the internal forces)
//    followed by the nodes themselves (weight 0), node a taking point NG + a:
//    tet10_nodal_stress (quadratic.rs:678-702), wedge6_nodal_stress
//    (extra.rs:134-153) and wedge15_nodal_stress (extra.rs:821-850) evaluate the
//    stress at the nodes.
struct RecTables {
  const double* dn;
  const double* w;
  const double* x;
  const int* perm;
};
struct NodeRecTab {
  double* dn = nullptr;
  double* w = nullptr;
  int device = -1;
};
NodeRecTab g_node_rec[3];  // tet10, wedge6, wedge15

// stiffness Gauss points of the element kinds whose stress is evaluated at the nodes
int node_eval_gauss(int nn) { return nn == 10 ? 4 : nn == 6 ? 6 : 9; }

// parametric positions of the nodes (tet10: quadratic.rs:680-691; wedges: extra.rs:137-144, 824-840)
std::vector<double> node_points(int nn) {
  if (nn == 10)
    return {0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1, 0.5, 0, 0, 0.5, 0.5, 0, 0, 0.5, 0, 0, 0, 0.5, 0.5, 0, 0.5, 0, 0.5, 0.5};
  std::vector<double> p = {1, 0, -1, 0, 1, -1, 0, 0, -1, 1, 0, 1, 0, 1, 1, 0, 0, 1};
  if (nn == 15) {
    const std::vector<double> mid = {0.5, 0.5, -1, 0, 0.5, -1, 0.5, 0, -1, 0.5, 0.5, 1, 0, 0.5, 1,
                                     0.5, 0,   1,  1, 0,   0,  0,   1, 0,  0,   0,   0};
    p.insert(p.end(), mid.begin(), mid.end());
  }
  return p;
}

int node_eval_index(int nn) { return nn == 10 ? 0 : nn == 6 ? 1 : 2; }

int ensure_xtab(axia_ctx* ctx, const double** x, const int** perm) {
  const int nn = ctx->nn;
  const int ti = nn == 4 ? 3 : nn == 10 ? 4 : nn == 6 ? 6 : nn == 15 ? 7 : (nn == 8 && ctx->ngp == 1) ? 5
               : nn == 8 ? 0 : (ctx->ngp == 27 ? 1 : 2);
  XTab& t = g_xtab[ti];
  if (t.device != ctx->device) {
    std::vector<double> hx;
    std::vector<int> hp;
    if (nn == 4 || (nn == 8 && ctx->ngp == 1)) {  // one point, every node takes its stress
      hx.assign(nn, 1.0);
      hp.assign(1, 0);
    } else if (nn == 10 || nn == 6 || nn == 15) {
      const int ng = node_eval_gauss(nn), np = ng + nn;
      hx.assign((size_t)nn * np, 0.0);
      for (int a = 0; a < nn; ++a) hx[(size_t)a * np + ng + a] = 1.0;
      hp.resize(np);
      for (int m = 0; m < np; ++m) hp[m] = m;
    } else {
      extrapolation_table(ctx->nn, ctx->ngp, hx, hp);
    }
    AXIA_CUDA(ctx, cudaMalloc(&t.x, hx.size() * sizeof(double)));
    AXIA_CUDA(ctx, cudaMalloc(&t.perm, hp.size() * sizeof(int)));
    AXIA_CUDA(ctx, cudaMemcpy(t.x, hx.data(), hx.size() * sizeof(double), cudaMemcpyHostToDevice));
    AXIA_CUDA(ctx, cudaMemcpy(t.perm, hp.data(), hp.size() * sizeof(int), cudaMemcpyHostToDevice));
    t.device = ctx->device;
  }
  *x = t.x;
  *perm = t.perm;
  return AXIA_OK;
}

int recover_tables(axia_ctx* ctx, RecTables* r) {
  AXIA_TRY(ensure_xtab(ctx, &r->x, &r->perm));
  const int nn = ctx->nn;
  if (nn != 10 && nn != 6 && nn != 15) return element_tables_for(ctx, nn, ctx->ngp, &r->dn, &r->w);
  NodeRecTab& t = g_node_rec[node_eval_index(nn)];
  if (t.device != ctx->device) {
    // the stiffness points and weights first, then the nodes with weight 0
    const double *gdn = nullptr, *gw = nullptr;
    const int ng = node_eval_gauss(nn), np = ng + nn;
    AXIA_TRY(element_tables_for(ctx, nn, ng, &gdn, &gw));
    std::vector<double> dn((size_t)np * nn * 3), w(np, 0.0);
    AXIA_CUDA(ctx, cudaMemcpy(dn.data(), gdn, (size_t)ng * nn * 3 * sizeof(double), cudaMemcpyDeviceToHost));
    AXIA_CUDA(ctx, cudaMemcpy(w.data(), gw, (size_t)ng * sizeof(double), cudaMemcpyDeviceToHost));
    const std::vector<double> pts = node_points(nn);
    for (int a = 0; a < nn; ++a)
      element_dshape(nn, pts[3 * a], pts[3 * a + 1], pts[3 * a + 2], &dn[(size_t)(ng + a) * nn * 3]);
    AXIA_CUDA(ctx, cudaMalloc(&t.dn, dn.size() * sizeof(double)));
    AXIA_CUDA(ctx, cudaMalloc(&t.w, w.size() * sizeof(double)));
    AXIA_CUDA(ctx, cudaMemcpy(t.dn, dn.data(), dn.size() * sizeof(double), cudaMemcpyHostToDevice));
    AXIA_CUDA(ctx, cudaMemcpy(t.w, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice));
    t.device = ctx->device;
  }
  r->dn = t.dn;
  r->w = t.w;
  return AXIA_OK;
}

template <int NN, int NG>
void launch_element_recover(axia_ctx* ctx, const double* d_u, const double* dn, const double* w, const double* xt,
                            const int* perm, double* d_emean) {
  using C = RecoverCfg<NN, NG>;
  const int64_t per_block = (int64_t)C::WARPS * C::EPW;
  const unsigned grid = (unsigned)std::max<int64_t>(
      1, std::min<int64_t>((ctx->n_elem + per_block - 1) / per_block, (int64_t)ctx->sm_count * 16));
  element_recover_kernel<NN, NG><<<grid, 32 * C::WARPS, 0, ctx->stream>>>(
      ctx->n_elem, ctx->d_conn, ctx->d_coords, d_u, ctx->d_e, ctx->nu, dn, w, xt, perm, ctx->d_rec, d_emean,
      ctx->d_status);
}

}  // namespace

// Device pointers, ordered on the context's stream.  Any output may be null.
int recover_device(axia_ctx* ctx, const double* d_u, const double* d_f, double e_strain, double* d_stress,
                   double* d_strain, double* d_vm, double* d_rf, double* d_emean) {
  if (!ctx->d_conn || !ctx->d_ne_ptr) return set_error(ctx, AXIA_ERR_STATE, "recovery before setup");
  if (ctx->nn == 8 && ctx->reduced && (!ctx->assembled || !ctx->d_ke))
    return set_error(ctx, AXIA_ERR_STATE, "recovery of C3D8R / C3D8I needs the assembled element stiffness");
  if (d_strain && !(e_strain > 0.0)) return set_error(ctx, AXIA_ERR_MATERIAL, "strain conversion needs E > 0");
  if (ctx->n_elem == 0) return AXIA_OK;
  if (!ctx->d_rec) AXIA_TRY(dev_alloc(ctx, &ctx->d_rec, (size_t)ctx->n_elem * ctx->nn * kRec));
  RecTables t{};
  AXIA_TRY(recover_tables(ctx, &t));
  AXIA_TRY(reset_dev_status(ctx));
  if (ctx->nn == 8 && ctx->ngp == 1)
    launch_element_recover<8, 1>(ctx, d_u, t.dn, t.w, t.x, t.perm, d_emean);
  else if (ctx->nn == 8)
    launch_element_recover<8, 8>(ctx, d_u, t.dn, t.w, t.x, t.perm, d_emean);
  else if (ctx->nn == 4)
    launch_element_recover<4, 1>(ctx, d_u, t.dn, t.w, t.x, t.perm, d_emean);
  else if (ctx->nn == 10)
    launch_element_recover<10, 14>(ctx, d_u, t.dn, t.w, t.x, t.perm, d_emean);
  else if (ctx->nn == 6)
    launch_element_recover<6, 12>(ctx, d_u, t.dn, t.w, t.x, t.perm, d_emean);
  else if (ctx->nn == 15)
    launch_element_recover<15, 24>(ctx, d_u, t.dn, t.w, t.x, t.perm, d_emean);
  else if (ctx->ngp == 27)
    launch_element_recover<20, 27>(ctx, d_u, t.dn, t.w, t.x, t.perm, d_emean);
  else
    launch_element_recover<20, 8>(ctx, d_u, t.dn, t.w, t.x, t.perm, d_emean);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  if (ctx->nn == 8 && ctx->reduced) {
    // C3D8R / C3D8I: the internal forces include the hourglass / condensed parts,
    // so they come from the assembled element stiffness: f_e = K_e u_e
    k_ke_force<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((ctx->n_elem + 3) / 4, ctx->sm_count * 16)), 128, 0,
                 ctx->stream>>>(ctx->n_elem, ctx->d_conn, ctx->d_ke, d_u, ctx->d_rec);
    ctx->launches++;
    AXIA_CUDA(ctx, cudaGetLastError());
  }
  const unsigned grid = (unsigned)std::max<int64_t>(
      1, std::min<int64_t>((ctx->n_nodes + 255) / 256, (int64_t)ctx->sm_count * 16));
  k_recover_nodes<<<grid, 256, 0, ctx->stream>>>(ctx->n_nodes, ctx->nn, ctx->d_ne_ptr, ctx->d_ne, ctx->d_rec, d_f,
                                                 ctx->nu, e_strain, d_stress, d_strain, d_vm, d_rf);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  DevStatus hs;
  AXIA_TRY(read_dev_status(ctx, &hs));
  if (hs.first_error != ~0ull) {
    ctx->last_bad = (int64_t)(hs.first_error >> 8);
    return set_error(ctx, (int)(hs.first_error & 0xff),
                     "stress recovery: element " + std::to_string(ctx->last_bad) + " invalid");
  }
  return AXIA_OK;
}

extern "C" {

int32_t axia_gpu_recover_device(axia_ctx* ctx, const double* u_full, const double* f_full, double e_strain,
                                double* stress, double* strain, double* vm, double* rf, double* elem_stress) {
  if (!ctx || !u_full) return AXIA_ERR_INVALID_ARG;
  AXIA_CUDA(ctx, cudaSetDevice(ctx->device));
  ctx->last_error.clear();
  return recover_device(ctx, u_full, f_full, e_strain, stress, strain, vm, rf, elem_stress);
}

int32_t axia_gpu_recover(axia_ctx* ctx, const double* u_full, const double* f_full, double e_strain, double* stress,
                         double* strain, double* vm, double* rf, double* elem_stress) {
  if (!ctx || !u_full) return AXIA_ERR_INVALID_ARG;
  AXIA_CUDA(ctx, cudaSetDevice(ctx->device));
  ctx->last_error.clear();
  if (!ctx->d_conn) return set_error(ctx, AXIA_ERR_STATE, "recovery before setup");
  const int64_t nd = ctx->ndof, nn6 = 6 * ctx->n_nodes, ne6 = 6 * ctx->n_elem;
  // one device block: u, f, stress, strain, vm, rf, element means
  const size_t total = (size_t)nd * 3 + (size_t)nn6 * 2 + ctx->n_nodes + ne6;
  double* buf = nullptr;
  AXIA_TRY(dev_alloc(ctx, &buf, std::max<size_t>(total, 1)));
  double* du = buf;
  double* df = du + nd;
  double* drf = df + nd;
  double* dst = drf + nd;
  double* dsn = dst + nn6;
  double* dvm = dsn + nn6;
  double* dem = dvm + ctx->n_nodes;
  int st = AXIA_OK;
  auto h2d = [&](double* d, const double* h, int64_t n) {
    if (st == AXIA_OK && cudaMemcpyAsync(d, h, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
      st = set_error(ctx, AXIA_ERR_CUDA, "copy to device");
  };
  auto d2h = [&](double* h, const double* d, int64_t n) {
    if (st == AXIA_OK && h && cudaMemcpyAsync(h, d, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess)
      st = set_error(ctx, AXIA_ERR_CUDA, "copy to host");
  };
  h2d(du, u_full, nd);
  if (f_full) h2d(df, f_full, nd);
  if (st == AXIA_OK)
    st = recover_device(ctx, du, f_full ? df : nullptr, e_strain, stress ? dst : nullptr, strain ? dsn : nullptr,
                        vm ? dvm : nullptr, rf ? drf : nullptr, elem_stress ? dem : nullptr);
  d2h(stress, dst, nn6);
  d2h(strain, dsn, nn6);
  d2h(vm, dvm, ctx->n_nodes);
  d2h(rf, drf, nd);
  d2h(elem_stress, dem, ne6);
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess && st == AXIA_OK)
    st = set_error(ctx, AXIA_ERR_CUDA, "stream synchronize after recovery");
  dev_free(buf);
  return st;
}

}  // extern "C"
