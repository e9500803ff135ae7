// pcg.cu -- persistent Jacobi-preconditioned CG on K_ff in CSR.
//
// Restates pcg (solver/src/linalg.rs:199-259): x0 = 0, z = r / diag with the
// |diag| > 1e-30 guard, stop at ||r||_2 <= tol ||b||_2, error when the final
// residual exceeds 10 tol ||b|| or |p.Ap| < 1e-30.  One cooperative launch runs
// every iteration: the SpMV q = K p with the p.q partial sum, the x / r update
// with the r.r and r.z partial sums, and the p update.  The two reductions are
// reduce-and-sync grid barriers (the last block to arrive sums all block
// partials in a fixed order and publishes the totals), the p update ends with
// a plain grid barrier; every wait is bounded.  Every block sees the same
// totals, takes the same branch, and results are bitwise reproducible.
//
// SpMV: L lanes per CSR row (vectorised CSR), matrix values and column
// indices loaded with evict-first hints so the vectors stay resident in L2.
//
// Mixed precision, two forms:
//  * restart: classic iterative refinement -- FP32 inner PCG on the FP32 copy
//    of K_ff to a residual reduction inner_rtol, FP64 update x += d and FP64
//    residual r = b - K_ff x, repeated (host loop, one launch per inner solve);
//  * reliable: one FP32 Krylov sequence in one launch; whenever its residual
//    has dropped by inner_rtol since the last update, the FP32 correction is
//    added to the FP64 solution and the FP32 residual is replaced by the FP64
//    residual b - K_ff x (search direction kept).  Convergence is decided on
//    the FP64 residual.
#include <algorithm>
#include <cmath>

#include "solver.cuh"

// One CSR row, L lanes: sum_k val[k] x[col[k]].
template <typename V, typename A, int L>
__device__ __forceinline__ A csr_row_dot(int row, int n, int sl, const int* __restrict__ rowptr,
                                         const int* __restrict__ col, const V* __restrict__ val, const V* x) {
  A s = 0;
  if (row < n) {
    const int beg = __ldg(rowptr + row), end = __ldg(rowptr + row + 1);
#pragma unroll 4
    for (int k = beg + sl; k < end; k += L) s = fma((A)ld_stream(val + k), (A)x[ld_stream(col + k)], s);
  }
  return group_sum<L>(s);
}

template <typename V, int L>
__global__ void __launch_bounds__(PCG_THREADS) pcg_kernel(PcgArgs<V> P) {
  using A = V;  // accumulation in the storage precision (FP64 or FP32)
  const int n = P.n;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nth = gridDim.x * blockDim.x;
  constexpr int RPW = 32 / L;  // rows per warp step
  const int gwarp = tid >> 5, nwarps = nth >> 5;
  const int lane = threadIdx.x & 31, sl = lane % L, grp = lane / L;

  // x = 0, r = b, z = r / diag, p = z
  A rz_p = 0, bb_p = 0;
  for (int i = tid; i < n; i += nth) {
    const V bi = P.b[i];
    P.x[i] = V(0);
    P.r[i] = bi;
    const V z = bi * P.dinv[i];
    P.p[i] = z;
    rz_p = fma(bi, z, rz_p);
    bb_p = fma(bi, bi, bb_p);
  }
  block_partials<A>(bb_p, rz_p, 2, P.partials, S_RR, S_RZ);
  double red[REDUCE_MAX_NV];
  if (!grid_reduce_sync(P.bar, P.st, P.limit_ns, P.partials, P.totals, S_RR, 2, red)) return;
  A rz = (A)red[1];
  const double bnorm = sqrt(red[0]);
  long long iters = 0;
  double residual = bnorm;
  int status = AXIA_OK;
  if (bnorm >= 1e-30) {
    for (long long it = 0; it < P.max_iter; ++it) {
      iters = it + 1;
      // q = K p, p.q
      A pq_p = 0;
      for (int base = gwarp * RPW; base < n; base += nwarps * RPW) {
        const int row = base + grp;
        const A s = csr_row_dot<V, A, L>(row, n, sl, P.rowptr, P.col, P.val, P.p);
        if (row < n && sl == 0) {
          P.q[row] = (V)s;
          pq_p = fma((A)P.p[row], s, pq_p);
        }
      }
      block_partials<A>(pq_p, A(0), 1, P.partials, S_PQ, S_PQ);
      double red[REDUCE_MAX_NV];
      if (!grid_reduce_sync(P.bar, P.st, P.limit_ns, P.partials, P.totals, S_PQ, 1, red)) return;
      const A pq = (A)red[0];
      if (!(fabs((double)pq) >= 1e-30)) {
        status = AXIA_ERR_ZERO_PIVOT;
        break;
      }
      const A alpha = rz / pq;
      // x += alpha p, r -= alpha q, r.r, r.z
      A rr_p = 0, rzn_p = 0;
      for (int i = tid; i < n; i += nth) {
        P.x[i] = fma(alpha, P.p[i], P.x[i]);
        const V ri = fma(-alpha, P.q[i], P.r[i]);
        P.r[i] = ri;
        rr_p = fma(ri, ri, rr_p);
        rzn_p = fma(ri, ri * P.dinv[i], rzn_p);
      }
      block_partials<A>(rr_p, rzn_p, 2, P.partials, S_RR, S_RZ);
      if (!grid_reduce_sync(P.bar, P.st, P.limit_ns, P.partials, P.totals, S_RR, 2, red)) return;
      const A rzn = (A)red[1];
      residual = sqrt(red[0]);
      if (!isfinite(residual)) {
        status = AXIA_ERR_NONFINITE;
        break;
      }
      if (residual <= P.tol * bnorm) break;
      const A beta = rzn / rz;
      rz = rzn;
      for (int i = tid; i < n; i += nth) P.p[i] = fma(beta, P.p[i], P.r[i] * P.dinv[i]);
      if (!grid_sync(P.bar, P.st, P.limit_ns)) return;
    }
    if (status == AXIA_OK && residual > P.tol * bnorm * 10.0) status = AXIA_ERR_NOT_CONVERGED;
  } else {
    residual = 0.0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    P.out->iters = iters;
    P.out->residual = residual;
    P.out->bnorm = bnorm;
    P.out->status = status;
    P.out->updates = 0;
  }
}

// ---------------------------------------------------------------------------
// Reliable-update mixed precision: FP32 CG on K32 with FP64 residual
// replacement (Sleijpen & van der Vorst's reliable updating, the scheme used
// for mixed-precision CG in lattice-QCD solvers).
// ---------------------------------------------------------------------------
struct ReliableArgs {
  int n;
  const int* rowptr;
  const int* col;
  const float* val32;
  const double* val64;
  const float* dinv32;
  const double* b;   // FP64 right-hand side
  double* x;         // FP64 solution
  double* r;         // FP64 residual (scratch)
  float* x32;        // FP32 correction since the last update
  float* r32;
  float* p32;
  float* q32;
  double* partials;
  double* totals;
  GridBarrier* bar;
  DevStatus* st;
  PcgOut* out;
  double tol;
  double delta;      // update when the FP32 residual fell by this factor
  long long max_iter;
  unsigned long long limit_ns;
};

template <int L32, int L64>
__global__ void __launch_bounds__(PCG_THREADS, 4) pcg_reliable_kernel(ReliableArgs P) {
  const int n = P.n;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nth = gridDim.x * blockDim.x;
  const int gwarp = tid >> 5, nwarps = nth >> 5;
  const int lane = threadIdx.x & 31;
  // x = 0, r32 = b, x32 = 0, p = z = r32 / diag
  float rz_p = 0.f;
  double bb_p = 0.0;
  for (int i = tid; i < n; i += nth) {
    const double bi = P.b[i];
    P.x[i] = 0.0;
    const float ri = (float)bi;
    P.r32[i] = ri;
    P.x32[i] = 0.f;
    const float z = ri * P.dinv32[i];
    P.p32[i] = z;
    rz_p = fmaf(ri, z, rz_p);
    bb_p = fma(bi, bi, bb_p);
  }
  block_partials<double>(bb_p, (double)rz_p, 2, P.partials, S_RR, S_RZ);
  double red[REDUCE_MAX_NV];
  if (!grid_reduce_sync(P.bar, P.st, P.limit_ns, P.partials, P.totals, S_RR, 2, red)) return;
  float rz = (float)red[1];
  const double bnorm = sqrt(red[0]);
  double rmax = bnorm;       // residual norm at the last update
  double residual = bnorm;   // FP64 residual norm at the last update
  long long iters = 0;
  int updates = 0, status = AXIA_OK;
  bool converged = bnorm < 1e-30;
  if (converged) residual = 0.0;
  for (long long it = 0; !converged && it < P.max_iter; ++it) {
    iters = it + 1;
    float pq_p = 0.f;
    {
      constexpr int RPW = 32 / L32;
      const int sl = lane % L32, grp = lane / L32;
      for (int base = gwarp * RPW; base < n; base += nwarps * RPW) {
        const int row = base + grp;
        const float s = csr_row_dot<float, float, L32>(row, n, sl, P.rowptr, P.col, P.val32, P.p32);
        if (row < n && sl == 0) {
          P.q32[row] = s;
          pq_p = fmaf(P.p32[row], s, pq_p);
        }
      }
    }
    block_partials<float>(pq_p, 0.f, 1, P.partials, S_PQ, S_PQ);
    double red[REDUCE_MAX_NV];
    if (!grid_reduce_sync(P.bar, P.st, P.limit_ns, P.partials, P.totals, S_PQ, 1, red)) return;
    const float pq = (float)red[0];
    if (!(fabsf(pq) >= 1e-30f) || !isfinite(pq)) {
      status = isfinite(pq) ? AXIA_ERR_ZERO_PIVOT : AXIA_ERR_NONFINITE;
      break;
    }
    const float alpha = rz / pq;
    float rr_p = 0.f, rzn_p = 0.f;
    for (int i = tid; i < n; i += nth) {
      P.x32[i] = fmaf(alpha, P.p32[i], P.x32[i]);
      const float ri = fmaf(-alpha, P.q32[i], P.r32[i]);
      P.r32[i] = ri;
      rr_p = fmaf(ri, ri, rr_p);
      rzn_p = fmaf(ri, ri * P.dinv32[i], rzn_p);
    }
    block_partials<float>(rr_p, rzn_p, 2, P.partials, S_RR, S_RZ);
    if (!grid_reduce_sync(P.bar, P.st, P.limit_ns, P.partials, P.totals, S_RR, 2, red)) return;
    float rzn = (float)red[1];
    const double rnorm32 = sqrt(red[0]);
    if (!isfinite(rnorm32)) {
      status = AXIA_ERR_NONFINITE;
      break;
    }
    if (rnorm32 <= P.delta * rmax || rnorm32 <= P.tol * bnorm) {
      // reliable update: x += x32 (FP64), r = b - K x (FP64), r32 = r
      for (int i = tid; i < n; i += nth) {
        P.x[i] += (double)P.x32[i];
        P.x32[i] = 0.f;
      }
      if (!grid_sync(P.bar, P.st, P.limit_ns)) return;
      double rr64_p = 0.0;
      float rz_new_p = 0.f;
      {
        constexpr int RPW = 32 / L64;
        const int sl = lane % L64, grp = lane / L64;
        for (int base = gwarp * RPW; base < n; base += nwarps * RPW) {
          const int row = base + grp;
          const double s = csr_row_dot<double, double, L64>(row, n, sl, P.rowptr, P.col, P.val64, P.x);
          if (row < n && sl == 0) {
            const double ri = P.b[row] - s;
            P.r[row] = ri;
            rr64_p = fma(ri, ri, rr64_p);
            const float r32 = (float)ri;
            P.r32[row] = r32;
            rz_new_p = fmaf(r32, r32 * P.dinv32[row], rz_new_p);
          }
        }
      }
      block_partials<double>(rr64_p, (double)rz_new_p, 2, P.partials, S_RR, S_RZ);
      double red[REDUCE_MAX_NV];
      if (!grid_reduce_sync(P.bar, P.st, P.limit_ns, P.partials, P.totals, S_RR, 2, red)) return;
      ++updates;
      residual = sqrt(red[0]);
      rzn = (float)red[1];
      rmax = residual;
      if (!isfinite(residual)) {
        status = AXIA_ERR_NONFINITE;
        break;
      }
      if (residual <= P.tol * bnorm) {
        converged = true;
        break;
      }
    }
    const float beta = rzn / rz;
    rz = rzn;
    for (int i = tid; i < n; i += nth) P.p32[i] = fmaf(beta, P.p32[i], P.r32[i] * P.dinv32[i]);
    if (!grid_sync(P.bar, P.st, P.limit_ns)) return;
  }
  if (status == AXIA_OK && residual > P.tol * bnorm * 10.0) status = AXIA_ERR_NOT_CONVERGED;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    P.out->iters = iters;
    P.out->residual = residual;
    P.out->bnorm = bnorm;
    P.out->status = status;
    P.out->updates = updates;
  }
}

// ---------------------------------------------------------------------------
// Helpers for refinement and the full-vector mapping
// ---------------------------------------------------------------------------
// r = b - K x (FP64), block partials of r.r into partials[blockIdx.x]
template <int L>
__global__ void __launch_bounds__(PCG_THREADS)
residual_kernel(int n, const int* rowptr, const int* col, const double* val, const double* b, const double* x,
                double* r, double* partials) {
  constexpr int RPW = 32 / L;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
  const int gwarp = tid >> 5, nwarps = nth >> 5;
  const int lane = threadIdx.x & 31, sl = lane % L, grp = lane / L;
  double rr = 0;
  for (int base = gwarp * RPW; base < n; base += nwarps * RPW) {
    const int row = base + grp;
    const double s = csr_row_dot<double, double, L>(row, n, sl, rowptr, col, val, x);
    if (row < n && sl == 0) {
      const double ri = b[row] - s;
      r[row] = ri;
      rr = fma(ri, ri, rr);
    }
  }
  block_partials<double>(rr, 0.0, 1, partials, 0, 0);
}

// y = K x, standalone (the matrix product of Csr::matvec, linalg.rs:41-50)
template <typename V, int L>
__global__ void __launch_bounds__(PCG_THREADS, 4)
spmv_kernel(int n, const int* rowptr, const int* col, const V* val, const V* x, V* y) {
  constexpr int RPW = 32 / L;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
  const int gwarp = tid >> 5, nwarps = nth >> 5;
  const int lane = threadIdx.x & 31, sl = lane % L, grp = lane / L;
  for (int base = gwarp * RPW; base < n; base += nwarps * RPW) {
    const int row = base + grp;
    const V s = csr_row_dot<V, V, L>(row, n, sl, rowptr, col, val, x);
    if (row < n && sl == 0) y[row] = s;
  }
}

template <typename V, int L>
static int launch_spmv_t(axia_ctx* ctx, const V* val, const V* x, V* y) {
  auto kern = spmv_kernel<V, L>;
  int per_sm = 0;
  AXIA_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, PCG_THREADS, 0));
  int grid = std::max(1, per_sm) * ctx->sm_count;
  kern<<<grid, PCG_THREADS, 0, ctx->stream>>>((int)ctx->n_free, ctx->d_rowptr, ctx->d_col, val, x, y);
  AXIA_CUDA(ctx, cudaGetLastError());
  ctx->launches++;
  return AXIA_OK;
}

template <typename V>
static int launch_spmv(axia_ctx* ctx, const V* val, const V* x, V* y, int lanes) {
  switch (lanes) {
    case 1: return launch_spmv_t<V, 1>(ctx, val, x, y);
    case 2: return launch_spmv_t<V, 2>(ctx, val, x, y);
    case 4: return launch_spmv_t<V, 4>(ctx, val, x, y);
    case 8: return launch_spmv_t<V, 8>(ctx, val, x, y);
    case 16: return launch_spmv_t<V, 16>(ctx, val, x, y);
    default: return launch_spmv_t<V, 32>(ctx, val, x, y);
  }
}

int spmv_device(axia_ctx* ctx, bool fp32, const void* x, void* y, int lanes_req) {
  const int lanes = pcg_lanes_for(ctx, fp32, lanes_req);
  if (fp32) return launch_spmv<float>(ctx, ctx->d_val32, (const float*)x, (float*)y, lanes);
  return launch_spmv<double>(ctx, ctx->d_val, (const double*)x, (double*)y, lanes);
}

__global__ void k_f64_to_f32(int n, const double* in, float* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = (float)in[i];
}
__global__ void k_add_f32_to_f64(int n, const float* d, double* x) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] += (double)d[i];
}

// rhs[r] = f[d] - K_fp u0 (reduce, constraint.rs:145-165)
__global__ void k_build_rhs(int64_t ndof, const int32_t* ind_of, const double* f, const double* kfu0, double* b) {
  for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < ndof; d += (int64_t)gridDim.x * blockDim.x) {
    const int r = ind_of[d];
    if (r >= 0) b[r] = f[d] - kfu0[r];
  }
}
// u = u0 + T x (reconstruct, constraint.rs:207-217)
__global__ void k_reconstruct(int64_t ndof, const int32_t* ind_of, const double* u0, const double* x, double* u) {
  for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < ndof; d += (int64_t)gridDim.x * blockDim.x) {
    const int r = ind_of[d];
    u[d] = r >= 0 ? u0[d] + x[r] : u0[d];
  }
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
// Lanes per CSR row.  FP64 work is scarce on GB300 (about 1/58 of the FP32
// rate), so the FP64 SpMV uses few lanes per row (fewer shuffle-add steps per
// row); the FP32 SpMV can afford wider groups for better coalescing.
static int pick_lanes(double avg_row, bool fp32) {
  if (fp32) {
    if (avg_row <= 12) return 4;
    if (avg_row <= 128) return 8;
    return 16;
  }
  if (avg_row <= 24) return 4;
  if (avg_row <= 160) return 8;
  return 16;
}

int pcg_lanes_for(const axia_ctx* ctx, bool fp32, int requested) {
  if (requested == 1 || requested == 2 || requested == 4 || requested == 8 || requested == 16 || requested == 32)
    return requested;
  double avg = ctx->n_free ? (double)ctx->nnz / (double)ctx->n_free : 1.0;
  return pick_lanes(avg, fp32);
}

template <typename V, int L>
static int launch_pcg_t(axia_ctx* ctx, PcgArgs<V>& P) {
  auto kern = pcg_kernel<V, L>;
  int grid = 0;
  AXIA_TRY(coop_grid(ctx, (const void*)kern, P.n, &grid));
  void* params[] = {&P};
  AXIA_CUDA(ctx, cudaLaunchCooperativeKernel((const void*)kern, dim3(grid), dim3(PCG_THREADS), params, 0, ctx->stream));
  ctx->launches++;
  return AXIA_OK;
}

template <typename V>
int launch_pcg(axia_ctx* ctx, PcgArgs<V>& P, int lanes) {
  switch (lanes) {
    case 1: return launch_pcg_t<V, 1>(ctx, P);
    case 2: return launch_pcg_t<V, 2>(ctx, P);
    case 4: return launch_pcg_t<V, 4>(ctx, P);
    case 8: return launch_pcg_t<V, 8>(ctx, P);
    case 16: return launch_pcg_t<V, 16>(ctx, P);
    default: return launch_pcg_t<V, 32>(ctx, P);
  }
}

template <int L32, int L64>
static int launch_reliable_t(axia_ctx* ctx, ReliableArgs& P) {
  auto kern = pcg_reliable_kernel<L32, L64>;
  int grid = 0;
  AXIA_TRY(coop_grid(ctx, (const void*)kern, P.n, &grid));
  void* params[] = {&P};
  AXIA_CUDA(ctx, cudaLaunchCooperativeKernel((const void*)kern, dim3(grid), dim3(PCG_THREADS), params, 0, ctx->stream));
  ctx->launches++;
  return AXIA_OK;
}

template <int L64>
static int launch_reliable_l32(axia_ctx* ctx, ReliableArgs& P, int l32) {
  switch (l32) {
    case 4: return launch_reliable_t<4, L64>(ctx, P);
    case 16: return launch_reliable_t<16, L64>(ctx, P);
    case 32: return launch_reliable_t<32, L64>(ctx, P);
    default: return launch_reliable_t<8, L64>(ctx, P);
  }
}

static int launch_reliable(axia_ctx* ctx, ReliableArgs& P, int l32, int l64) {
  switch (l64) {
    case 2: return launch_reliable_l32<2>(ctx, P, l32);
    case 8: return launch_reliable_l32<8>(ctx, P, l32);
    default: return launch_reliable_l32<4>(ctx, P, l32);
  }
}

static int ensure_solver_buffers(axia_ctx* ctx, bool mixed) {
  const size_t n = (size_t)ctx->n_free;
  if (ctx->vec_capacity < n || (mixed && !ctx->d_x32)) {
    AXIA_TRY(dev_alloc(ctx, &ctx->d_b, n));
    AXIA_TRY(dev_alloc(ctx, &ctx->d_x, n));
    AXIA_TRY(dev_alloc(ctx, &ctx->d_r, n));
    AXIA_TRY(dev_alloc(ctx, &ctx->d_p, n));
    AXIA_TRY(dev_alloc(ctx, &ctx->d_q, n));
    if (mixed) {
      AXIA_TRY(dev_alloc(ctx, &ctx->d_b32, n));
      AXIA_TRY(dev_alloc(ctx, &ctx->d_x32, n));
      AXIA_TRY(dev_alloc(ctx, &ctx->d_r32, n));
      AXIA_TRY(dev_alloc(ctx, &ctx->d_p32, n));
      AXIA_TRY(dev_alloc(ctx, &ctx->d_q32, n));
    }
    ctx->vec_capacity = n;
  }
  return AXIA_OK;
}

static double residual_norm(axia_ctx* ctx, const double* b, const double* x, double* r) {
  const int n = (int)ctx->n_free;
  int grid = ctx->sm_count * 4;
  int lanes = pcg_lanes_for(ctx, false, 0);
  ctx->launches++;
  switch (lanes) {
    case 8: residual_kernel<8><<<grid, PCG_THREADS, 0, ctx->stream>>>(n, ctx->d_rowptr, ctx->d_col, ctx->d_val, b, x, r, ctx->d_partials); break;
    default: residual_kernel<4><<<grid, PCG_THREADS, 0, ctx->stream>>>(n, ctx->d_rowptr, ctx->d_col, ctx->d_val, b, x, r, ctx->d_partials); break;
  }
  std::vector<double> h(grid);
  cudaMemcpyAsync(h.data(), ctx->d_partials, grid * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  double s = 0.0;
  for (double v : h) s += v;
  return std::sqrt(s);
}

// Solves K_ff x = b (d_b) into d_x.  Fills info fields iters / outer / residual / bnorm.
int pcg_solve(axia_ctx* ctx, const axia_solve_opts* opts, axia_solve_info* info) {
  const bool mixed = opts->precision == AXIA_PREC_MIXED;
  if (mixed && !ctx->have32) return set_error(ctx, AXIA_ERR_STATE, "mixed precision needs axia_gpu_assemble(AXIA_PREC_MIXED)");
  AXIA_TRY(ensure_solver_buffers(ctx, mixed));
  AXIA_TRY(reset_dev_status(ctx));
  const int n = (int)ctx->n_free;
  const long long max_iter = opts->max_iter > 0 ? opts->max_iter : std::max<long long>(4LL * n, 200);
  const int lanes = pcg_lanes_for(ctx, mixed, opts->spmv_lanes);
  const unsigned long long limit_ns = 2000000000ull;  // 2 s per barrier wait
  AXIA_CUDA(ctx, cudaMemsetAsync(ctx->d_bar, 0, sizeof(GridBarrier), ctx->stream));
  PcgOut o{};
  if (!mixed) {
    PcgArgs<double> P{n, ctx->d_rowptr, ctx->d_col, ctx->d_val, ctx->d_dinv, ctx->d_b, ctx->d_x, ctx->d_r, ctx->d_p,
                      ctx->d_q, ctx->d_partials, ctx->d_totals, ctx->d_bar, ctx->d_status, (PcgOut*)ctx->d_out,
                      opts->rtol, max_iter, limit_ns};
    AXIA_TRY(timed_launch(ctx, info, [&] { return launch_pcg<double>(ctx, P, lanes); }));
    AXIA_TRY(read_out(ctx, &o));
    info->iters = o.iters;
    info->outer_iters = 1;
    info->residual = o.residual;
    info->bnorm = o.bnorm;
    if (o.status != AXIA_OK) return status_error(ctx, o);
    return AXIA_OK;
  }
  if (opts->refine_mode == AXIA_REFINE_RELIABLE) {
    const double delta = opts->inner_rtol > 0 && opts->inner_rtol < 1 ? opts->inner_rtol : 0.1;
    ReliableArgs P{n, ctx->d_rowptr, ctx->d_col, ctx->d_val32, ctx->d_val, ctx->d_dinv32, ctx->d_b, ctx->d_x,
                   ctx->d_r, ctx->d_x32, ctx->d_r32, ctx->d_p32, ctx->d_q32, ctx->d_partials, ctx->d_totals,
                   ctx->d_bar, ctx->d_status, (PcgOut*)ctx->d_out, opts->rtol, delta, max_iter, limit_ns};
    const int l64 = pcg_lanes_for(ctx, false, 0);
    AXIA_TRY(timed_launch(ctx, info, [&] { return launch_reliable(ctx, P, lanes, l64); }));
    AXIA_TRY(read_out(ctx, &o));
    info->iters = o.iters;
    info->outer_iters = o.updates;
    info->residual = o.residual;
    info->bnorm = o.bnorm;
    if (o.status != AXIA_OK) return status_error(ctx, o);
    return AXIA_OK;
  }
  // restart: FP64 iterative refinement around an FP32 PCG on K32
  const int tb = 256, gb = ctx->sm_count * 8;
  AXIA_CUDA(ctx, cudaMemsetAsync(ctx->d_x, 0, n * sizeof(double), ctx->stream));
  double bnorm = residual_norm(ctx, ctx->d_b, ctx->d_x, ctx->d_r);  // x = 0: r = b, ||b||
  info->bnorm = bnorm;
  info->iters = 0;
  info->outer_iters = 0;
  double rnorm = bnorm;
  if (bnorm < 1e-30) {
    info->residual = 0.0;
    return AXIA_OK;
  }
  const int max_outer = opts->max_outer > 0 ? opts->max_outer : 50;
  const double inner = opts->inner_rtol > 0 ? opts->inner_rtol : 1e-3;
  for (int outer = 0; outer < max_outer && rnorm > opts->rtol * bnorm; ++outer) {
    k_f64_to_f32<<<gb, tb, 0, ctx->stream>>>(n, ctx->d_r, ctx->d_b32);
    ctx->launches++;
    AXIA_CUDA(ctx, cudaMemsetAsync(ctx->d_bar, 0, sizeof(GridBarrier), ctx->stream));
    // inner tolerance: the requested reduction, but no tighter than needed to reach rtol
    double itol = std::max(inner, 0.5 * opts->rtol * bnorm / rnorm);
    PcgArgs<float> P{n, ctx->d_rowptr, ctx->d_col, ctx->d_val32, ctx->d_dinv32, ctx->d_b32, ctx->d_x32, ctx->d_r32,
                     ctx->d_p32, ctx->d_q32, ctx->d_partials, ctx->d_totals, ctx->d_bar, ctx->d_status,
                     (PcgOut*)ctx->d_out, itol, max_iter, limit_ns};
    AXIA_TRY(timed_launch(ctx, info, [&] { return launch_pcg<float>(ctx, P, lanes); }));
    AXIA_TRY(read_out(ctx, &o));
    info->iters += o.iters;
    info->outer_iters = outer + 1;
    if (o.status == AXIA_ERR_ZERO_PIVOT || o.status == AXIA_ERR_NONFINITE)
      return set_error(ctx, o.status, "mixed-precision inner CG broke down");
    k_add_f32_to_f64<<<gb, tb, 0, ctx->stream>>>(n, ctx->d_x32, ctx->d_x);
    ctx->launches++;
    rnorm = residual_norm(ctx, ctx->d_b, ctx->d_x, ctx->d_r);
    if (!std::isfinite(rnorm)) return set_error(ctx, AXIA_ERR_NONFINITE, "non-finite residual in refinement");
  }
  info->residual = rnorm;
  if (rnorm > opts->rtol * bnorm * 10.0)
    return set_error(ctx, AXIA_ERR_NOT_CONVERGED, "refinement did not converge (residual " + std::to_string(rnorm) + ")");
  return AXIA_OK;
}

int true_residual(axia_ctx* ctx, double* out) {
  *out = residual_norm(ctx, ctx->d_b, ctx->d_x, ctx->d_q);
  return AXIA_OK;
}

int prepare_solve(axia_ctx* ctx, bool mixed) { return ensure_solver_buffers(ctx, mixed); }

int build_rhs(axia_ctx* ctx, const double* d_f) {
  if (!ctx->d_b || !ctx->d_kfu0 || !ctx->d_ind_of || !d_f)
    return set_error(ctx, AXIA_ERR_STATE, "right-hand side buffers not allocated");
  k_build_rhs<<<ctx->sm_count * 8, 256, 0, ctx->stream>>>(ctx->ndof, ctx->d_ind_of, d_f, ctx->d_kfu0, ctx->d_b);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  return AXIA_OK;
}

int reconstruct(axia_ctx* ctx, double* d_u) {
  if (!ctx->d_x || !ctx->d_u0 || !d_u) return set_error(ctx, AXIA_ERR_STATE, "solution buffers not allocated");
  k_reconstruct<<<ctx->sm_count * 8, 256, 0, ctx->stream>>>(ctx->ndof, ctx->d_ind_of, ctx->d_u0, ctx->d_x, d_u);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  return AXIA_OK;
}

int ensure_pcg_state(axia_ctx* ctx) {
  if (!ctx->d_partials) {
    ctx->partial_slots = (size_t)64 * 2048;  // up to 64 reduction slots x 2048 blocks
    AXIA_TRY(dev_alloc(ctx, &ctx->d_partials, ctx->partial_slots));
  }
  if (!ctx->d_totals) AXIA_TRY(dev_alloc(ctx, &ctx->d_totals, 64));
  if (!ctx->d_bar) AXIA_TRY(dev_alloc(ctx, &ctx->d_bar, 1));
  if (!ctx->d_out) {
    PcgOut* o = nullptr;
    AXIA_TRY(dev_alloc(ctx, &o, 1));
    ctx->d_out = o;
  }
  return AXIA_OK;
}
