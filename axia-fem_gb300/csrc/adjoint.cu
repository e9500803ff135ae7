// adjoint.cu -- compliance and its gradient for a SIMP density field.
//
// No reference counterpart: the reference has no adjoint or sensitivity code.
// Model: E_e = E0 rho_e^p, compliance C = f . u with K(rho) u = f.  Because K
// is self-adjoint the adjoint solution is -u and
//   dC/drho_e = -p rho_e^(p-1) E0 u_e^T K_e(E=1) u_e .
// The element kernel evaluates the bilinear element form s_e = u_e^T K_e(1) v_e
// matrix-free at the Gauss points of the reference's element
// (hex8_stiffness solver/src/elem.rs:194-219, hex20_stiffness
// solver/src/quadratic.rs:122-146, tetrahedra and wedges likewise):
//   s_e = sum_gp w det J [lam tr(eps_u) tr(eps_v) + 2 mu eps_u:eps_v + mu gam_u.gam_v]
// (Voigt, engineering shears: the isotropic D of d_iso_3d, elem.rs:41-59, at E=1).
// Lanes are (element, Gauss point) pairs, 32/NG elements per warp, so every
// lane does FP64 work; the Gauss-point sums are segmented warp reductions.
#include <algorithm>
#include <cmath>
#include <vector>

#include "solver.cuh"

int element_tables_for(axia_ctx* ctx, int nn, int ng, const double** dn, const double** w);

template <int NN, int NG>
__global__ void __launch_bounds__(NN == 8 ? 256 : 128)
element_energy_kernel(int64_t n_elem, const int32_t* __restrict__ conn, const double* __restrict__ coords,
                      const double* __restrict__ u, const double* __restrict__ v, const double* __restrict__ dn_tab,
                      const double* __restrict__ w_tab, double c_lam, double c_mu, double* __restrict__ s_out,
                      DevStatus* st) {
  constexpr int EPW = 32 / NG;      // elements per warp step
  constexpr int ND = 3 * NN;
  constexpr int WARPS = NN == 8 ? 8 : 4;
  __shared__ double s_dn[NG * NN * 3];
  __shared__ double s_w[NG];
  __shared__ double s_x[WARPS][EPW][ND];
  __shared__ double s_u[WARPS][EPW][ND];
  __shared__ double s_v[WARPS][EPW][ND];
  for (int t = threadIdx.x; t < NG * NN * 3; t += blockDim.x) s_dn[t] = dn_tab[t];
  for (int t = threadIdx.x; t < NG; t += blockDim.x) s_w[t] = w_tab[t];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int le = lane / NG, g = lane % NG;
  const bool active_lane = le < EPW;
  const int64_t step = (int64_t)gridDim.x * WARPS * EPW;
  for (int64_t e0 = ((int64_t)blockIdx.x * WARPS + warp) * EPW; e0 < n_elem; e0 += step) {
    for (int t = lane; t < EPW * ND; t += 32) {
      const int k = t / ND, c = t % ND;
      const int64_t e = e0 + k;
      double xv = 0.0, uv = 0.0, vv = 0.0;
      if (e < n_elem) {
        const int64_t node = conn[e * NN + c / 3];
        xv = coords[3 * node + c % 3];
        uv = u[3 * node + c % 3];
        vv = v[3 * node + c % 3];
      }
      s_x[warp][k][c] = xv;
      s_u[warp][k][c] = uv;
      s_v[warp][k][c] = vv;
    }
    __syncwarp();
    double contrib = 0.0;
    const int64_t e = e0 + le;
    if (active_lane && e < n_elem) {
      const double* X = s_x[warp][le];
      const double* U = s_u[warp][le];
      const double* Vv = s_v[warp][le];
      const double* dn = s_dn + g * NN * 3;
      double J[3][3] = {}, Gu[3][3] = {}, Gv[3][3] = {};
#pragma unroll 4
      for (int a = 0; a < NN; ++a) {
        const double d0 = dn[3 * a], d1 = dn[3 * a + 1], d2 = dn[3 * a + 2];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          const double xq = X[3 * a + q], uq = U[3 * a + q], vq = Vv[3 * a + q];
          J[q][0] = fma(d0, xq, J[q][0]);
          J[q][1] = fma(d1, xq, J[q][1]);
          J[q][2] = fma(d2, xq, J[q][2]);
          Gu[0][q] = fma(d0, uq, Gu[0][q]);
          Gu[1][q] = fma(d1, uq, Gu[1][q]);
          Gu[2][q] = fma(d2, uq, Gu[2][q]);
          Gv[0][q] = fma(d0, vq, Gv[0][q]);
          Gv[1][q] = fma(d1, vq, Gv[1][q]);
          Gv[2][q] = fma(d2, vq, Gv[2][q]);
        }
      }
      // cofactors b[i][j] (inverse = b / det, invert3 elem.rs:10-29)
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
      } else if (det <= 0.0) {
        record_error(st, e, AXIA_ERR_NEG_JACOBIAN);
      }
      // det * du_q/dx_i = sum_p b[p][i] Gu[p][q]  (kept scaled by det)
      double Hu[3][3], Hv[3][3];
#pragma unroll
      for (int q = 0; q < 3; ++q)
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          Hu[q][i] = fma(b[0][i], Gu[0][q], fma(b[1][i], Gu[1][q], b[2][i] * Gu[2][q]));
          Hv[q][i] = fma(b[0][i], Gv[0][q], fma(b[1][i], Gv[1][q], b[2][i] * Gv[2][q]));
        }
      const double tru = Hu[0][0] + Hu[1][1] + Hu[2][2], trv = Hv[0][0] + Hv[1][1] + Hv[2][2];
      const double nn_ = Hu[0][0] * Hv[0][0] + Hu[1][1] * Hv[1][1] + Hu[2][2] * Hv[2][2];
      const double gg = (Hu[0][1] + Hu[1][0]) * (Hv[0][1] + Hv[1][0]) + (Hu[1][2] + Hu[2][1]) * (Hv[1][2] + Hv[2][1]) +
                        (Hu[2][0] + Hu[0][2]) * (Hv[2][0] + Hv[0][2]);
      const double dens = c_lam * tru * trv + 2.0 * c_mu * nn_ + c_mu * gg;  // det^2 * energy density
      contrib = s_w[g] * dens / det;                                         // w det * density
    }
    // segmented sum over the NG lanes of each element
    if constexpr ((NG & (NG - 1)) == 0) {
#pragma unroll
      for (int o = NG / 2; o > 0; o >>= 1) contrib += __shfl_xor_sync(0xffffffffu, contrib, o);
    } else if constexpr (EPW == 1) {
      contrib = warp_sum(contrib);  // one element per warp
    } else {
      // lane le * NG sums its element's NG lanes in order (C3D6: 5 x 6, C3D15: 3 x 9)
      double t = contrib;
#pragma unroll
      for (int k = 1; k < NG; ++k) t += __shfl_down_sync(0xffffffffu, contrib, k);
      contrib = t;
    }
    if (active_lane && g == 0 && e < n_elem) s_out[e] = contrib;
    __syncwarp();
  }
}

// C3D8R / C3D8I: s_e = u_e^T K_e v_e / E_e from the assembled element stiffness (the
// hourglass and condensed parts are linear in E too); one warp per element
__global__ void k_ke_energy(int64_t n_elem, const int32_t* __restrict__ conn, const double* __restrict__ ke,
                            const double* __restrict__ e_elem, const double* __restrict__ u,
                            const double* __restrict__ v, double* __restrict__ s_out) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t e = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); e < n_elem; e += warps) {
    const int64_t d = lane < 24 ? 3 * (int64_t)conn[e * 8 + lane / 3] + lane % 3 : 0;
    const double ve = lane < 24 ? v[d] : 0.0, ue = lane < 24 ? u[d] : 0.0;
    double kv = 0.0;
    const double* row = ke + e * 576 + (int64_t)(lane < 24 ? lane : 0) * 24;
    for (int j = 0; j < 24; ++j) kv = fma(row[j], __shfl_sync(0xffffffffu, ve, j), kv);
    const double t = warp_sum(lane < 24 ? ue * kv : 0.0);
    if (lane == 0) s_out[e] = t / e_elem[e];
  }
}

// E_e = e0 rho_e^p
__global__ void k_simp_modulus(int64_t n, const double* rho, double pexp, double e0, double* e_out, DevStatus* st) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double r = rho[i];
    if (!(r > 0.0) || !isfinite(r)) record_error(st, i, AXIA_ERR_MATERIAL);
    e_out[i] = e0 * pow(r, pexp);
  }
}

// g_e = -p rho_e^(p-1) e0 s_e
__global__ void k_simp_gradient(int64_t n, const double* rho, const double* s, double pexp, double e0, double* g) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    g[i] = -pexp * pow(rho[i], pexp - 1.0) * e0 * s[i];
}

// f . u in a fixed order: per-block partials, summed on the host in block order
__global__ void k_dot_partials(int64_t n, const double* a, const double* b, double* partials) {
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s = fma(a[i], b[i], s);
  __shared__ double red[32];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    t = warp_sum(t);
    if (threadIdx.x == 0) partials[blockIdx.x] = t;
  }
}

int element_energy(axia_ctx* ctx, const double* d_u, const double* d_v, double* d_s) {
  const double c_lam = ctx->nu / ((1.0 + ctx->nu) * (1.0 - 2.0 * ctx->nu));
  const double c_mu = 1.0 / (2.0 * (1.0 + ctx->nu));
  const double *dn = nullptr, *w = nullptr;
  AXIA_TRY(element_tables_for(ctx, ctx->nn, ctx->ngp, &dn, &w));
  AXIA_TRY(reset_dev_status(ctx));
  if (ctx->nn == 8 && ctx->reduced) {
    if (!ctx->assembled || !ctx->d_ke)
      return set_error(ctx, AXIA_ERR_STATE, "element energy of C3D8R / C3D8I needs the assembled element stiffness");
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((ctx->n_elem + 3) / 4, ctx->sm_count * 16));
    k_ke_energy<<<grid, 128, 0, ctx->stream>>>(ctx->n_elem, ctx->d_conn, ctx->d_ke, ctx->d_e, d_u, d_v, d_s);
  } else if (ctx->nn == 8) {
    const int threads = 256;
    const int64_t per_block = 8 * 4;
    const unsigned grid = (unsigned)std::min<int64_t>((ctx->n_elem + per_block - 1) / per_block, ctx->sm_count * 16);
    element_energy_kernel<8, 8><<<std::max(1u, grid), threads, 0, ctx->stream>>>(
        ctx->n_elem, ctx->d_conn, ctx->d_coords, d_u, d_v, dn, w, c_lam, c_mu, d_s, ctx->d_status);
  } else if (ctx->nn == 4) {
    const int threads = 128;
    const int64_t per_block = 4 * 32;
    const unsigned grid = (unsigned)std::min<int64_t>((ctx->n_elem + per_block - 1) / per_block, ctx->sm_count * 16);
    element_energy_kernel<4, 1><<<std::max(1u, grid), threads, 0, ctx->stream>>>(
        ctx->n_elem, ctx->d_conn, ctx->d_coords, d_u, d_v, dn, w, c_lam, c_mu, d_s, ctx->d_status);
  } else if (ctx->nn == 10) {
    const int threads = 128;
    const int64_t per_block = 4 * 8;
    const unsigned grid = (unsigned)std::min<int64_t>((ctx->n_elem + per_block - 1) / per_block, ctx->sm_count * 16);
    element_energy_kernel<10, 4><<<std::max(1u, grid), threads, 0, ctx->stream>>>(
        ctx->n_elem, ctx->d_conn, ctx->d_coords, d_u, d_v, dn, w, c_lam, c_mu, d_s, ctx->d_status);
  } else if (ctx->nn == 6 || ctx->nn == 15) {
    const int threads = 128;
    const int64_t per_block = 4 * (ctx->nn == 6 ? 32 / 6 : 32 / 9);
    const unsigned grid = (unsigned)std::min<int64_t>((ctx->n_elem + per_block - 1) / per_block, ctx->sm_count * 16);
    if (ctx->nn == 6)
      element_energy_kernel<6, 6><<<std::max(1u, grid), threads, 0, ctx->stream>>>(
          ctx->n_elem, ctx->d_conn, ctx->d_coords, d_u, d_v, dn, w, c_lam, c_mu, d_s, ctx->d_status);
    else
      element_energy_kernel<15, 9><<<std::max(1u, grid), threads, 0, ctx->stream>>>(
          ctx->n_elem, ctx->d_conn, ctx->d_coords, d_u, d_v, dn, w, c_lam, c_mu, d_s, ctx->d_status);
  } else if (ctx->ngp == 27) {
    const int threads = 128;
    const int64_t per_block = 4;
    const unsigned grid = (unsigned)std::min<int64_t>((ctx->n_elem + per_block - 1) / per_block, ctx->sm_count * 16);
    element_energy_kernel<20, 27><<<std::max(1u, grid), threads, 0, ctx->stream>>>(
        ctx->n_elem, ctx->d_conn, ctx->d_coords, d_u, d_v, dn, w, c_lam, c_mu, d_s, ctx->d_status);
  } else {
    const int threads = 128;
    const int64_t per_block = 4 * 4;
    const unsigned grid = (unsigned)std::min<int64_t>((ctx->n_elem + per_block - 1) / per_block, ctx->sm_count * 16);
    element_energy_kernel<20, 8><<<std::max(1u, grid), threads, 0, ctx->stream>>>(
        ctx->n_elem, ctx->d_conn, ctx->d_coords, d_u, d_v, dn, w, c_lam, c_mu, d_s, ctx->d_status);
  }
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  DevStatus hs;
  AXIA_TRY(read_dev_status(ctx, &hs));
  if (hs.first_error != ~0ull) {
    ctx->last_bad = (int64_t)(hs.first_error >> 8);
    return set_error(ctx, (int)(hs.first_error & 0xff), "element " + std::to_string(ctx->last_bad) + ": invalid element");
  }
  return AXIA_OK;
}

int simp_modulus(axia_ctx* ctx, const double* d_rho, double pexp, double e0) {
  AXIA_TRY(reset_dev_status(ctx));
  k_simp_modulus<<<ctx->sm_count * 4, 256, 0, ctx->stream>>>(ctx->n_elem, d_rho, pexp, e0, ctx->d_e, ctx->d_status);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  DevStatus hs;
  AXIA_TRY(read_dev_status(ctx, &hs));
  if (hs.first_error != ~0ull) {
    ctx->last_bad = (int64_t)(hs.first_error >> 8);
    return set_error(ctx, AXIA_ERR_MATERIAL, "density of element " + std::to_string(ctx->last_bad) + " not positive");
  }
  return AXIA_OK;
}

int simp_gradient(axia_ctx* ctx, const double* d_rho, const double* d_s, double pexp, double e0, double* d_g) {
  k_simp_gradient<<<ctx->sm_count * 4, 256, 0, ctx->stream>>>(ctx->n_elem, d_rho, d_s, pexp, e0, d_g);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  return AXIA_OK;
}

int device_dot(axia_ctx* ctx, const double* a, const double* b, int64_t n, double* out) {
  const int grid = ctx->sm_count * 2;
  k_dot_partials<<<grid, 256, 0, ctx->stream>>>(n, a, b, ctx->d_partials);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  std::vector<double> h(grid);
  AXIA_CUDA(ctx, cudaMemcpyAsync(h.data(), ctx->d_partials, grid * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  double s = 0.0;
  for (double v : h) s += v;
  *out = s;
  return AXIA_OK;
}
