// Host check of the element-stiffness arithmetic of the double-word kernels
// (axia-fem_gb300/csrc/element_dw.cuh): the closed form
//   K_ab = lam A_ab + mu A_ab^T + mu tr(A_ab) I,  A_ab = sum_g (w / det J) c_a c_b^T,
//   c_a = adj(J)^T dN_a / dxi,
// evaluated with the primitives of dword.cuh in the kernels' order
// (coordinates relative to node 0 and scaled by 2^-k, J, cofactors, det,
// w / det, c, h = (w / det) c, A, traces, K), against an independent
// long-double stiffness of the textbook form
//   K = sum_g w det J B^T D B with dN/dx = J^-T dN/dxi
// for C3D8 (2x2x2 Gauss points) and C3D20 (3x3x3), on distorted elements of
// edge 1e-3 .. 1e3 placed up to 100 edges from the origin.  The split of the
// scaled coordinates into double words rounds to nearest here (the kernels
// truncate: the same 48 significant bits).  Prints the worst error per kind
// and exits non-zero when one exceeds 1e-13 of max|Ke|.
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "../../axia-fem_gb300/csrc/dword.cuh"

typedef long double R;

struct Kind {
  int nn, ng;
  std::vector<double> xi;  // [nn][3] natural coordinates of the nodes
  std::vector<double> gp;  // [ng][3]
  std::vector<double> gw;  // [ng]
};

// dN_a/dxi_p at natural point (x, y, z): 8-node trilinear, or 20-node serendipity
static void dshape(const Kind& k, double x, double y, double z, std::vector<double>& dn) {
  dn.assign((size_t)k.nn * 3, 0.0);
  for (int a = 0; a < k.nn; ++a) {
    const double xa = k.xi[3 * a], ya = k.xi[3 * a + 1], za = k.xi[3 * a + 2];
    const double sx = 1 + x * xa, sy = 1 + y * ya, sz = 1 + z * za;
    double* d = &dn[3 * a];
    if (k.nn == 8) {
      d[0] = 0.125 * xa * sy * sz;
      d[1] = 0.125 * ya * sx * sz;
      d[2] = 0.125 * za * sx * sy;
    } else if (xa != 0 && ya != 0 && za != 0) {  // corner: N = (1/8) sx sy sz (x xa + y ya + z za - 2)
      const double t = x * xa + y * ya + z * za - 2;
      d[0] = 0.125 * (xa * sy * sz * t + sx * sy * sz * xa);
      d[1] = 0.125 * (ya * sx * sz * t + sx * sy * sz * ya);
      d[2] = 0.125 * (za * sx * sy * t + sx * sy * sz * za);
    } else if (xa == 0) {  // mid-edge along x: N = (1/4) (1 - x^2) sy sz
      d[0] = 0.25 * (-2 * x) * sy * sz;
      d[1] = 0.25 * (1 - x * x) * ya * sz;
      d[2] = 0.25 * (1 - x * x) * sy * za;
    } else if (ya == 0) {
      d[0] = 0.25 * (1 - y * y) * xa * sz;
      d[1] = 0.25 * (-2 * y) * sx * sz;
      d[2] = 0.25 * (1 - y * y) * sx * za;
    } else {
      d[0] = 0.25 * (1 - z * z) * xa * sy;
      d[1] = 0.25 * (1 - z * z) * sx * ya;
      d[2] = 0.25 * (-2 * z) * sx * sy;
    }
  }
}

static Kind make_kind(int nn) {
  Kind k;
  k.nn = nn;
  const int c[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                       {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
  for (int a = 0; a < 8; ++a)
    for (int d = 0; d < 3; ++d) k.xi.push_back(c[a][d]);
  if (nn == 20) {  // the twelve edge midpoints
    const int e[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6}, {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
    for (auto& p : e)
      for (int d = 0; d < 3; ++d) k.xi.push_back(0.5 * (c[p[0]][d] + c[p[1]][d]));
  }
  const int m = nn == 8 ? 2 : 3;
  const double g2 = 1.0 / std::sqrt(3.0), g3 = std::sqrt(0.6);
  const double pts[3] = {-(m == 2 ? g2 : g3), m == 2 ? g2 : 0.0, g3};
  const double wts[3] = {m == 2 ? 1.0 : 5.0 / 9.0, m == 2 ? 1.0 : 8.0 / 9.0, 5.0 / 9.0};
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j)
      for (int l = 0; l < m; ++l) {
        k.gp.push_back(pts[i]);
        k.gp.push_back(pts[j]);
        k.gp.push_back(pts[l]);
        k.gw.push_back(wts[i] * wts[j] * wts[l]);
      }
  k.ng = (int)k.gw.size();
  return k;
}

// long double B^T D B stiffness (isotropic D in Voigt form written out)
static std::vector<R> ke_ref(const Kind& k, const std::vector<double>& X, double E, double nu) {
  const int nd = 3 * k.nn;
  std::vector<R> K((size_t)nd * nd, 0);
  const R lam = (R)E * nu / ((1 + (R)nu) * (1 - 2 * (R)nu)), mu = (R)E / (2 * (1 + (R)nu));
  std::vector<double> dn;
  for (int g = 0; g < k.ng; ++g) {
    dshape(k, k.gp[3 * g], k.gp[3 * g + 1], k.gp[3 * g + 2], dn);
    R J[3][3] = {};
    for (int a = 0; a < k.nn; ++a)
      for (int q = 0; q < 3; ++q)
        for (int p = 0; p < 3; ++p) J[q][p] += (R)dn[3 * a + p] * (R)X[3 * a + q];
    const R det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                  J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    R Ji[3][3];  // inverse of J (J[q][p] = dx_q / dxi_p): Ji[p][q] = dxi_p / dx_q
    Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
    Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
    Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
    Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
    Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
    Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
    Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
    Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
    std::vector<R> dx((size_t)k.nn * 3, 0);  // dN_a/dx_i = sum_p dN_a/dxi_p dxi_p/dx_i
    for (int a = 0; a < k.nn; ++a)
      for (int i = 0; i < 3; ++i)
        for (int p = 0; p < 3; ++p) dx[3 * a + i] += (R)dn[3 * a + p] * Ji[p][i];
    const R f = (R)k.gw[g] * det;
    for (int a = 0; a < k.nn; ++a)
      for (int b = 0; b < k.nn; ++b) {
        const R* da = &dx[3 * a];
        const R* db = &dx[3 * b];
        const R dot = da[0] * db[0] + da[1] * db[1] + da[2] * db[2];
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j)
            K[(size_t)(3 * a + i) * nd + 3 * b + j] += f * (lam * da[i] * db[j] + mu * da[j] * db[i] + (i == j ? mu * dot : 0));
      }
  }
  return K;
}

// the double-word closed form in the kernels' order
static std::vector<double> ke_dw(const Kind& k, const std::vector<double>& X, double E, double nu) {
  const int nn = k.nn, nd = 3 * nn, ng = k.ng;
  int emax = 0;
  std::vector<double> dif(nd);
  for (int t = 0; t < nd; ++t) {
    dif[t] = X[t] - X[t % 3];
    int e;
    if (dif[t] != 0) {
      std::frexp(dif[t], &e);
      emax = std::max(emax, e + 1022);
    }
  }
  const int kx = emax == 0 ? 0 : emax - 1022;  // |dif| < 2^kx
  std::vector<dw> Xw(nd);
  for (int t = 0; t < nd; ++t) Xw[t] = dw_from_double(std::ldexp(dif[t], -kx));
  std::vector<dw> C((size_t)ng * nd), H((size_t)ng * nd);
  std::vector<double> dn;
  for (int g = 0; g < ng; ++g) {
    dshape(k, k.gp[3 * g], k.gp[3 * g + 1], k.gp[3 * g + 2], dn);
    std::vector<dw> dnw(nd);
    for (int t = 0; t < nd; ++t) dnw[t] = dw_from_double(dn[t]);
    dw J[9], G[9];
    for (int t = 0; t < 9; ++t) {  // J[q][p] = sum_a dN_a/dxi_p x_a,q
      const int q = t / 3, p = t % 3;
      dw_acc s;
      for (int a = 0; a < nn; ++a) dw_fma(s, dnw[3 * a + p], Xw[3 * a + q]);
      J[t] = dw_value(s);
    }
    for (int t = 0; t < 9; ++t) {  // cofactors b[i][j]
      const int i = t / 3, j = t % 3;
      const int j1 = (j + 1) % 3, j2 = (j + 2) % 3, i1 = (i + 1) % 3, i2 = (i + 2) % 3;
      dw_acc s;
      dw_fma(s, J[3 * j1 + i1], J[3 * j2 + i2]);
      dw_fma(s, dw_neg(J[3 * j1 + i2]), J[3 * j2 + i1]);
      G[t] = dw_value(s);
    }
    dw_acc sd;
    dw_fma(sd, J[0], G[0]);
    dw_fma(sd, J[1], G[3]);
    dw_fma(sd, J[2], G[6]);
    const dw S = dw_div(dw_from_double(k.gw[g]), dw_value(sd));
    for (int r = 0; r < nd; ++r) {  // c_a[i] = sum_p b[p][i] dN_a/dxi_p, h = S c
      const int a = r / 3, i = r % 3;
      dw_acc s;
      dw_fma(s, G[i], dnw[3 * a]);
      dw_fma(s, G[3 + i], dnw[3 * a + 1]);
      dw_fma(s, G[6 + i], dnw[3 * a + 2]);
      C[(size_t)g * nd + r] = dw_value(s);
      H[(size_t)g * nd + r] = dw_mul(S, C[(size_t)g * nd + r]);
    }
  }
  const double c_lam = nu / ((1 + nu) * (1 - 2 * nu)), c_mu = 1 / (2 * (1 + nu));
  const dw Ew = dw_from_double(E);
  auto scale = [&](dw v) { return dw{(float)std::ldexp(v.h, kx), (float)std::ldexp(v.l, kx)}; };
  const dw lam = scale(dw_mul(Ew, dw_from_double(c_lam))), mu = scale(dw_mul(Ew, dw_from_double(c_mu)));
  std::vector<double> K((size_t)nd * nd);
  for (int a = 0; a < nn; ++a)
    for (int b = a; b < nn; ++b) {
      dw A[9];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          dw_acc s;
          for (int g = 0; g < ng; ++g) dw_fma(s, H[(size_t)g * nd + 3 * a + i], C[(size_t)g * nd + 3 * b + j]);
          A[3 * i + j] = dw_value(s);
        }
      dw_acc ts;
      dw_add(ts, A[0]);
      dw_add(ts, A[4]);
      dw_add(ts, A[8]);
      const dw tr = dw_value(ts);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          if (a == b && i > j) continue;
          dw_acc s;
          dw_fma(s, lam, A[3 * i + j]);
          dw_fma(s, mu, A[3 * j + i]);
          if (i == j) dw_fma(s, mu, tr);
          const double v = dw_to_double(dw_value(s));
          K[(size_t)(3 * a + i) * nd + 3 * b + j] = v;
          K[(size_t)(3 * b + j) * nd + 3 * a + i] = v;
        }
    }
  return K;
}

int main() {
  std::mt19937_64 rng(20261204);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  int fails = 0;
  for (int nn : {8, 20}) {
    const Kind k = make_kind(nn);
    // the shape derivatives themselves (both forms share them): sum_a dN_a/dxi_p = 0
    // and sum_a dN_a/dxi_p xi_a,q = delta_pq at every Gauss point
    std::vector<double> dn;
    double shape_err = 0;
    for (int g = 0; g < k.ng; ++g) {
      dshape(k, k.gp[3 * g], k.gp[3 * g + 1], k.gp[3 * g + 2], dn);
      for (int p = 0; p < 3; ++p) {
        double s0 = 0, s1[3] = {0, 0, 0};
        for (int a = 0; a < nn; ++a) {
          s0 += dn[3 * a + p];
          for (int q = 0; q < 3; ++q) s1[q] += dn[3 * a + p] * k.xi[3 * a + q];
        }
        shape_err = std::max(shape_err, std::fabs(s0));
        for (int q = 0; q < 3; ++q) shape_err = std::max(shape_err, std::fabs(s1[q] - (p == q)));
      }
    }
    std::printf("C3D%d: shape derivatives, partition of unity and linear completeness: %.1e\n", nn, shape_err);
    if (!(shape_err <= 1e-14)) ++fails;
    double worst = 0;
    for (double size : {1e-3, 0.05, 1.0, 1e3})
      for (double offset : {0.0, 2.0, 100.0}) {
        for (int rep = 0; rep < 12; ++rep) {
          double sc[3], sh[3];
          for (int d = 0; d < 3; ++d) {
            sc[d] = size * (0.5 + 1.5 * U(rng));
            sh[d] = offset * size * (2 * U(rng) - 1);
          }
          const double amp = 0.08 * std::min(sc[0], std::min(sc[1], sc[2]));
          std::vector<double> X((size_t)3 * nn);
          for (int a = 0; a < nn; ++a)
            for (int d = 0; d < 3; ++d)
              X[3 * a + d] = 0.5 * (k.xi[3 * a + d] + 1) * sc[d] + amp * (2 * U(rng) - 1) + sh[d];
          const double E = 1e3 + U(rng) * 2e11;
          const std::vector<R> ref = ke_ref(k, X, E, 0.3);
          const std::vector<double> got = ke_dw(k, X, E, 0.3);
          R mx = 0, err = 0;
          for (size_t t = 0; t < ref.size(); ++t) {
            mx = std::max(mx, std::fabs(ref[t]));
            err = std::max(err, std::fabs((R)got[t] - ref[t]));
          }
          worst = std::max(worst, (double)(err / mx));
        }
      }
    std::printf("C3D%d: worst |Ke_dw - Ke| / max|Ke| = %.3e\n", nn, worst);
    if (!(worst <= 1e-13)) ++fails;
  }
  return fails ? 1 : 0;
}
