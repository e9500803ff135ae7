// hex8_variants.cu -- the C3D8R and C3D8I parts of the element stiffness.
//
// C3D8R (solver/src/extra.rs:400-457): the one-point stiffness
// 8 det(J0) B0^T D B0 comes from element_ke_kernel<8, 1, .> (the centre
// point with weight 8); k_hex8r_hourglass then adds the Flanagan-Belytschko
// hourglass stiffness: for the four hourglass base vectors h_alpha,
//   gamma_alpha,a = h_alpha,a - sum_j (sum_b h_alpha,b x_b,j) dN_a/dx_j (centre),
//   K[(3a+d),(3b+d)] += q_alpha gamma_alpha,a gamma_alpha,b,
//   q_alpha = 0.1 mu vol^(1/3) / |gamma_alpha|^2 (skipped if |gamma|^2 < 1e-30),
// added for alpha = 0..3 in turn as the reference does.
//
// C3D8I (extra.rs:256-388): the compatible stiffness Kee comes from the
// standard 2x2x2 kernel; k_hex8i_condense adds the nine incompatible modes
// (gradients of 1 - xi_m^2 mapped with the centre Jacobian, g_m = -2 xi_m
// J0^-T e_m) and condenses them: Kaa = sum_gp det Ba^T D Ba (9x9),
// Kea = sum_gp det Be^T D Ba (24x9), Ke -= Kea Kaa^-1 Kea^T, with Kaa^-1 by
// Gauss-Jordan elimination with partial pivoting (invert_n, extra.rs:8-49;
// a pivot below 1e-18 is reported as a singular element).  For the isotropic
// D the 3x3 block of two gradient vectors p, r is
//   lam p_i r_j + mu p_j r_i + mu delta_ij (p . r).
// One warp per element; the small matrices live in shared memory.
#include <cmath>

#include "element.cuh"

namespace {

__constant__ double c_hourglass[4][8] = {{1, -1, 1, -1, 1, -1, 1, -1},  // extra.rs:413-418
                                          {1, 1, -1, -1, -1, -1, 1, 1},
                                          {1, -1, -1, 1, -1, 1, 1, -1},
                                          {-1, 1, -1, 1, 1, -1, 1, -1}};
__constant__ double c_hex_xi[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                      {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};

__device__ __forceinline__ double elem_coord(const ElemArgs& A, int64_t e, int a, int q) {
  if (A.conn) return A.coords[3 * (int64_t)A.conn[e * 8 + a] + q];
  return A.xyz[(e * 8 + a) * 3 + q];
}

// J0 (centre), its cofactors b (inverse = b / det) and det; dN_a/dxi at the centre = HEX_XI_a / 8
__device__ __forceinline__ double centre_jacobian(const double x[8][3], double b[3][3]) {
  double J[3][3] = {};
  for (int a = 0; a < 8; ++a)
    for (int p = 0; p < 3; ++p)
      for (int q = 0; q < 3; ++q) J[q][p] = fma(0.125 * c_hex_xi[a][p], x[a][q], J[q][p]);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      const int j1 = (j + 1) % 3, j2 = (j + 2) % 3, i1 = (i + 1) % 3, i2 = (i + 2) % 3;
      b[i][j] = J[j1][i1] * J[j2][i2] - J[j1][i2] * J[j2][i1];
    }
  return J[0][0] * b[0][0] + J[0][1] * b[1][0] + J[0][2] * b[2][0];
}

// one thread per element: hourglass stiffness added to the element's Ke (row-major 24x24)
__global__ void k_hex8r_hourglass(ElemArgs A) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < A.n_elem; e += (int64_t)gridDim.x * blockDim.x) {
    double x[8][3];
    for (int a = 0; a < 8; ++a)
      for (int q = 0; q < 3; ++q) x[a][q] = elem_coord(A, e, a, q);
    double b[3][3];
    const double det = centre_jacobian(x, b);
    if (!(fabs(det) >= 1e-18) || det <= 0.0) continue;  // reported by the element kernel
    const double inv = 1.0 / det;
    double dndx[8][3];
    for (int a = 0; a < 8; ++a)
      for (int i = 0; i < 3; ++i)
        dndx[a][i] = (b[0][i] * c_hex_xi[a][0] + b[1][i] * c_hex_xi[a][1] + b[2][i] * c_hex_xi[a][2]) * 0.125 * inv;
    const double E = A.e_elem ? A.e_elem[e] : A.e_const;
    const double mu = E * A.c_mu;
    const double vol = 8.0 * det;
    const double coeff = 0.1 * mu * pow(vol, 1.0 / 3.0);
    double* ke = A.ke_out + e * 576;
    for (int al = 0; al < 4; ++al) {
      double hx[3] = {0.0, 0.0, 0.0};
      for (int a = 0; a < 8; ++a)
        for (int j = 0; j < 3; ++j) hx[j] = fma(c_hourglass[al][a], x[a][j], hx[j]);
      double g[8], g2 = 0.0;
      for (int a = 0; a < 8; ++a) {
        g[a] = c_hourglass[al][a] - hx[0] * dndx[a][0] - hx[1] * dndx[a][1] - hx[2] * dndx[a][2];
        g2 = fma(g[a], g[a], g2);
      }
      if (g2 < 1e-30) continue;
      const double q = coeff / g2;
      for (int a = 0; a < 8; ++a)
        for (int bn = 0; bn < 8; ++bn) {
          const double v = q * g[a] * g[bn];
          for (int d = 0; d < 3; ++d) ke[(3 * a + d) * 24 + 3 * bn + d] += v;
        }
    }
  }
}

constexpr int kCondWarps = 4;
// per warp: x 24, dndx*det per gp 8*24, det 8, g per gp 8*9, Kea 216, Kaa 81 (+ aug 81), T 216
constexpr int kCondDoubles = 24 + 192 + 8 + 72 + 216 + 162 + 216;

__global__ void __launch_bounds__(32 * kCondWarps) k_hex8i_condense(ElemArgs A, const double* __restrict__ dn_tab) {
  __shared__ double s_dn[8 * 8 * 3];
  __shared__ double s_mem[kCondWarps][kCondDoubles];
  for (int t = threadIdx.x; t < 192; t += blockDim.x) s_dn[t] = dn_tab[t];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* X = s_mem[warp];      // [8][3]
  double* DX = X + 24;          // [8 gp][8 node][3]: det * dN/dx (= cofactor contraction)
  double* DET = DX + 192;       // [8]
  double* G = DET + 8;          // [8 gp][3 mode][3]: g_m at each gp (same J0 for all gp)
  double* KEA = G + 72;         // [24][9]
  double* AUG = KEA + 216;      // [9][18]: Kaa | I, reduced in place to I | Kaa^-1
  double* T = AUG + 162;        // [9][24]: Kaa^-1 Kea^T
  const double lam_c = A.c_lam, mu_c = A.c_mu;
  for (int64_t e = (int64_t)blockIdx.x * kCondWarps + warp; e < A.n_elem; e += (int64_t)gridDim.x * kCondWarps) {
    if (lane < 24) X[lane] = elem_coord(A, e, lane / 3, lane % 3);
    __syncwarp();
    const double E = A.e_elem ? A.e_elem[e] : A.e_const;
    const double lam = E * lam_c, mu = E * mu_c;
    // per Gauss point (lanes 0..7): J, cofactors, det; det * dN/dx; mode gradients
    if (lane < 8) {
      const int g = lane;
      const double* dn = s_dn + g * 24;
      double J[3][3] = {};
      for (int a = 0; a < 8; ++a)
        for (int p = 0; p < 3; ++p)
          for (int q = 0; q < 3; ++q) J[q][p] = fma(dn[3 * a + p], X[3 * a + q], J[q][p]);
      double b[3][3];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          const int j1 = (j + 1) % 3, j2 = (j + 2) % 3, i1 = (i + 1) % 3, i2 = (i + 2) % 3;
          b[i][j] = J[j1][i1] * J[j2][i2] - J[j1][i2] * J[j2][i1];
        }
      const double det = J[0][0] * b[0][0] + J[0][1] * b[1][0] + J[0][2] * b[2][0];
      DET[g] = det;
      for (int a = 0; a < 8; ++a)
        for (int i = 0; i < 3; ++i)
          DX[g * 24 + 3 * a + i] = b[0][i] * dn[3 * a] + b[1][i] * dn[3 * a + 1] + b[2][i] * dn[3 * a + 2];
      // centre Jacobian inverse (the same for every gp): inv0 = b0 / det0
      double x8[8][3];
      for (int a = 0; a < 8; ++a)
        for (int q = 0; q < 3; ++q) x8[a][q] = X[3 * a + q];
      double b0[3][3];
      const double det0 = centre_jacobian(x8, b0);
      const double inv0 = 1.0 / det0;
      // xi_m of this gp: the tables run xi, eta, zeta from - to + (xi outermost)
      const double g2 = 0.5773502691896257;
      const double xi_m[3] = {(g & 4) ? g2 : -g2, (g & 2) ? g2 : -g2, (g & 1) ? g2 : -g2};
      for (int m = 0; m < 3; ++m)
        for (int i = 0; i < 3; ++i) G[g * 9 + 3 * m + i] = (b0[m][i] * inv0) * (-2.0 * xi_m[m]);
    }
    __syncwarp();
    // Kea[(3a+i)][(3m+j)] = sum_gp det [lam dndx_a,i g_m,j + mu dndx_a,j g_m,i + mu delta_ij dndx_a . g_m]
    for (int t = lane; t < 216; t += 32) {
      const int r = t / 9, c = t % 9, a = r / 3, i = r % 3, m = c / 3, j = c % 3;
      double s = 0.0;
      for (int g = 0; g < 8; ++g) {
        const double* dx = DX + g * 24 + 3 * a;  // det * dN_a/dx
        const double* gm = G + g * 9 + 3 * m;
        double v = lam * dx[i] * gm[j] + mu * dx[j] * gm[i];
        if (i == j) v += mu * (dx[0] * gm[0] + dx[1] * gm[1] + dx[2] * gm[2]);
        s += v;
      }
      KEA[t] = s;
    }
    // Kaa (left half of AUG) and the identity (right half)
    for (int t = lane; t < 162; t += 32) {
      const int r = t / 18, c = t % 18;
      double s = 0.0;
      if (c < 9) {
        const int m = r / 3, i = r % 3, n = c / 3, j = c % 3;
        for (int g = 0; g < 8; ++g) {
          const double* gm = G + g * 9 + 3 * m;
          const double* gn = G + g * 9 + 3 * n;
          double v = lam * gm[i] * gn[j] + mu * gm[j] * gn[i];
          if (i == j) v += mu * (gm[0] * gn[0] + gm[1] * gn[1] + gm[2] * gn[2]);
          s = fma(DET[g], v, s);
        }
      } else {
        s = (c - 9 == r) ? 1.0 : 0.0;
      }
      AUG[t] = s;
    }
    __syncwarp();
    // Gauss-Jordan with partial pivoting; lane j < 18 owns column j
    int singular = 0;
    for (int k = 0; k < 9; ++k) {
      int piv = k;
      double best = fabs(AUG[k * 18 + k]);
      for (int i = k + 1; i < 9; ++i) {
        const double v = fabs(AUG[i * 18 + k]);
        if (v > best) {
          best = v;
          piv = i;
        }
      }
      if (best < 1e-18) {
        singular = 1;
        break;
      }
      if (piv != k && lane < 18) {
        const double t0 = AUG[k * 18 + lane];
        AUG[k * 18 + lane] = AUG[piv * 18 + lane];
        AUG[piv * 18 + lane] = t0;
      }
      __syncwarp();
      const double dkk = AUG[k * 18 + k];
      __syncwarp();
      if (lane < 18) AUG[k * 18 + lane] /= dkk;
      __syncwarp();
      double f[9];
      for (int i = 0; i < 9; ++i) f[i] = AUG[i * 18 + k];
      __syncwarp();
      if (lane < 18)
        for (int i = 0; i < 9; ++i)
          if (i != k) AUG[i * 18 + lane] -= f[i] * AUG[k * 18 + lane];
      __syncwarp();
    }
    if (singular) {
      if (lane == 0) record_error(A.status, e, AXIA_ERR_SINGULAR_JACOBIAN);
      __syncwarp();
      continue;
    }
    // T = Kaa^-1 Kea^T (9 x 24)
    for (int t = lane; t < 216; t += 32) {
      const int i = t / 24, j = t % 24;
      double s = 0.0;
      for (int k = 0; k < 9; ++k) s += AUG[i * 18 + 9 + k] * KEA[j * 9 + k];
      T[t] = s;
    }
    __syncwarp();
    double* ke = A.ke_out + e * 576;
    for (int t = lane; t < 576; t += 32) {
      const int i = t / 24, j = t % 24;
      double s = 0.0;
      for (int k = 0; k < 9; ++k) s += KEA[i * 9 + k] * T[k * 24 + j];
      ke[t] -= s;
    }
    __syncwarp();
  }
}

}  // namespace

int run_hex8r_hourglass(axia_ctx* ctx, const ElemArgs& args) {
  const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((args.n_elem + 127) / 128, ctx->sm_count * 8));
  k_hex8r_hourglass<<<grid, 128, 0, ctx->stream>>>(args);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  return AXIA_OK;
}

int run_hex8i_condense(axia_ctx* ctx, const ElemArgs& args, const double* dn_tab) {
  const unsigned grid =
      (unsigned)std::max<int64_t>(1, std::min<int64_t>((args.n_elem + kCondWarps - 1) / kCondWarps, ctx->sm_count * 16));
  k_hex8i_condense<<<grid, 32 * kCondWarps, 0, ctx->stream>>>(args, dn_tab);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  return AXIA_OK;
}
