// pcg.cu -- persistent Jacobi-preconditioned CG on K_ff in CSR.
//
// Restates pcg (solver/src/linalg.rs:199-259): x0 = 0, z = r / diag with the
// |diag| > 1e-30 guard, stop at ||r||_2 <= tol ||b||_2, error when the final
// residual exceeds 10 tol ||b|| or |p.Ap| < 1e-30.  One cooperative launch runs
// every iteration: the SpMV q = K p with the p.q partial sum, the x / r update
// with the r.r and r.z partial sums, and the p update, separated by three
// bounded grid barriers.  Dot products are reduced per block and then summed
// by every block over all block partials in a fixed order, so every block
// takes the same branch and the result is bitwise reproducible.
//
// SpMV: L lanes per row (vectorised CSR), matrix values and column indices
// loaded with evict-first hints so the vectors stay resident in L2.
#include <algorithm>
#include <cmath>

#include "common.cuh"

constexpr int PCG_THREADS = 256;
int pcg_lanes_for(const axia_ctx* ctx, bool fp32, int requested);
constexpr int S_PQ = 0, S_RR = 1, S_RZ = 2, N_SLOTS = 3;

struct PcgOut {
  long long iters;
  double residual;
  double bnorm;
  int status;
  int pad;
};

template <typename V>
struct PcgArgs {
  int n;
  const int* rowptr;
  const int* col;
  const V* val;
  const V* dinv;
  const V* b;
  V* x;
  V* r;
  V* p;
  V* q;
  double* partials;  // [N_SLOTS][gridDim.x]
  GridBarrier* bar;
  DevStatus* st;
  PcgOut* out;
  double tol;
  long long max_iter;
  unsigned long long limit_ns;
};

template <int L, typename T>
__device__ __forceinline__ T group_sum(T v) {
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block-reduce up to two values and store them as this block's partials
template <typename A>
__device__ __forceinline__ void block_partials(A v0, A v1, int nv, double* partials, int slot0, int slot1) {
  __shared__ A s_red[2][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  v0 = warp_sum(v0);
  if (nv > 1) v1 = warp_sum(v1);
  if (lane == 0) {
    s_red[0][warp] = v0;
    s_red[1][warp] = v1;
  }
  __syncthreads();
  if (warp == 0) {
    A a0 = lane < nw ? s_red[0][lane] : A(0);
    A a1 = lane < nw ? s_red[1][lane] : A(0);
    a0 = warp_sum(a0);
    if (nv > 1) a1 = warp_sum(a1);
    if (lane == 0) {
      partials[slot0 * gridDim.x + blockIdx.x] = (double)a0;
      if (nv > 1) partials[slot1 * gridDim.x + blockIdx.x] = (double)a1;
    }
  }
}

// sum of all block partials of a slot, same order in every block
template <typename A>
__device__ __forceinline__ void grid_sums(const double* partials, int slot0, int slot1, int nv, A* r0, A* r1) {
  __shared__ A s_out[2];
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    A a0 = 0, a1 = 0;
    for (int k = lane; k < (int)gridDim.x; k += 32) {
      a0 += (A)__ldcg(partials + slot0 * gridDim.x + k);
      if (nv > 1) a1 += (A)__ldcg(partials + slot1 * gridDim.x + k);
    }
    a0 = warp_sum(a0);
    if (nv > 1) a1 = warp_sum(a1);
    if (lane == 0) {
      s_out[0] = a0;
      s_out[1] = a1;
    }
  }
  __syncthreads();
  *r0 = s_out[0];
  if (nv > 1) *r1 = s_out[1];
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
  block_partials<A>(rz_p, bb_p, 2, P.partials, S_RZ, S_RR);
  if (!grid_sync(P.bar, P.st, P.limit_ns)) return;
  A rz, bb;
  grid_sums<A>(P.partials, S_RZ, S_RR, 2, &rz, &bb);
  const double bnorm = sqrt((double)bb);
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
        A s = 0;
        if (row < n) {
          const int beg = __ldg(P.rowptr + row), end = __ldg(P.rowptr + row + 1);
          for (int k = beg + sl; k < end; k += L) s = fma((A)ld_stream(P.val + k), (A)P.p[ld_stream(P.col + k)], s);
        }
        s = group_sum<L>(s);
        if (row < n && sl == 0) {
          P.q[row] = (V)s;
          pq_p = fma((A)P.p[row], s, pq_p);
        }
      }
      block_partials<A>(pq_p, A(0), 1, P.partials, S_PQ, S_PQ);
      if (!grid_sync(P.bar, P.st, P.limit_ns)) return;
      A pq;
      grid_sums<A>(P.partials, S_PQ, S_PQ, 1, &pq, &pq);
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
      if (!grid_sync(P.bar, P.st, P.limit_ns)) return;
      A rr, rzn;
      grid_sums<A>(P.partials, S_RR, S_RZ, 2, &rr, &rzn);
      residual = sqrt((double)rr);
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
    double s = 0;
    if (row < n) {
      const int beg = __ldg(rowptr + row), end = __ldg(rowptr + row + 1);
      for (int k = beg + sl; k < end; k += L) s = fma(ld_stream(val + k), x[ld_stream(col + k)], s);
    }
    s = group_sum<L>(s);
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
__global__ void __launch_bounds__(PCG_THREADS)
spmv_kernel(int n, const int* rowptr, const int* col, const V* val, const V* x, V* y) {
  constexpr int RPW = 32 / L;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
  const int gwarp = tid >> 5, nwarps = nth >> 5;
  const int lane = threadIdx.x & 31, sl = lane % L, grp = lane / L;
  for (int base = gwarp * RPW; base < n; base += nwarps * RPW) {
    const int row = base + grp;
    V s = 0;
    if (row < n) {
      const int beg = __ldg(rowptr + row), end = __ldg(rowptr + row + 1);
      for (int k = beg + sl; k < end; k += L) s = fma(ld_stream(val + k), __ldg(x + ld_stream(col + k)), s);
    }
    s = group_sum<L>(s);
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
  if (avg_row <= 48) return 4;
  if (avg_row <= 160) return 4;
  return 8;
}

int pcg_lanes_for(const axia_ctx* ctx, bool fp32, int requested) {
  if (requested == 4 || requested == 8 || requested == 16 || requested == 32) return requested;
  double avg = ctx->n_free ? (double)ctx->nnz / (double)ctx->n_free : 1.0;
  return pick_lanes(avg, fp32);
}

template <typename V, int L>
static int launch_pcg_t(axia_ctx* ctx, PcgArgs<V>& P) {
  auto kern = pcg_kernel<V, L>;
  int per_sm = 0;
  AXIA_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, PCG_THREADS, 0));
  if (per_sm < 1) return set_error(ctx, AXIA_ERR_CUDA, "PCG kernel does not fit on an SM");
  int grid = per_sm * ctx->sm_count;
  int need = (P.n + PCG_THREADS - 1) / PCG_THREADS;
  grid = std::max(1, std::min(grid, std::max(need, ctx->sm_count)));
  if ((size_t)grid * N_SLOTS > ctx->partial_slots) return set_error(ctx, AXIA_ERR_STATE, "partials buffer too small");
  void* params[] = {&P};
  AXIA_CUDA(ctx, cudaLaunchCooperativeKernel((const void*)kern, dim3(grid), dim3(PCG_THREADS), params, 0, ctx->stream));
  ctx->launches++;
  return AXIA_OK;
}

template <typename V>
int launch_pcg(axia_ctx* ctx, PcgArgs<V>& P, int lanes) {
  switch (lanes) {
    case 4: return launch_pcg_t<V, 4>(ctx, P);
    case 8: return launch_pcg_t<V, 8>(ctx, P);
    case 16: return launch_pcg_t<V, 16>(ctx, P);
    default: return launch_pcg_t<V, 32>(ctx, P);
  }
}

// one persistent PCG launch bracketed by CUDA events on the launching stream
template <typename V>
static int timed_pcg(axia_ctx* ctx, PcgArgs<V>& P, int lanes, axia_solve_info* info) {
  cudaEvent_t a, b;
  AXIA_CUDA(ctx, cudaEventCreate(&a));
  AXIA_CUDA(ctx, cudaEventCreate(&b));
  cudaEventRecord(a, ctx->stream);
  int st = launch_pcg<V>(ctx, P, lanes);
  cudaEventRecord(b, ctx->stream);
  if (st == AXIA_OK) {
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    info->ms_pcg_kernel += ms;
    info->pcg_launches += 1;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return st;
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

static int read_out(axia_ctx* ctx, PcgOut* o) {
  AXIA_CUDA(ctx, cudaMemcpyAsync(o, ctx->d_out, sizeof(PcgOut), cudaMemcpyDeviceToHost, ctx->stream));
  AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  DevStatus hs;
  AXIA_TRY(read_dev_status(ctx, &hs));
  if (hs.timeout) return set_error(ctx, AXIA_ERR_TIMEOUT, "a grid barrier of the PCG kernel ran past its time limit");
  return AXIA_OK;
}

static double residual_norm(axia_ctx* ctx, const double* b, const double* x, double* r) {
  const int n = (int)ctx->n_free;
  int grid = ctx->sm_count * 4;
  int lanes = pcg_lanes_for(ctx, false, 0);
  ctx->launches++;
  switch (lanes) {
    case 4: residual_kernel<4><<<grid, PCG_THREADS, 0, ctx->stream>>>(n, ctx->d_rowptr, ctx->d_col, ctx->d_val, b, x, r, ctx->d_partials); break;
    case 8: residual_kernel<8><<<grid, PCG_THREADS, 0, ctx->stream>>>(n, ctx->d_rowptr, ctx->d_col, ctx->d_val, b, x, r, ctx->d_partials); break;
    case 16: residual_kernel<16><<<grid, PCG_THREADS, 0, ctx->stream>>>(n, ctx->d_rowptr, ctx->d_col, ctx->d_val, b, x, r, ctx->d_partials); break;
    default: residual_kernel<32><<<grid, PCG_THREADS, 0, ctx->stream>>>(n, ctx->d_rowptr, ctx->d_col, ctx->d_val, b, x, r, ctx->d_partials); break;
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
                      ctx->d_q, ctx->d_partials, ctx->d_bar, ctx->d_status, (PcgOut*)ctx->d_out, opts->rtol, max_iter,
                      limit_ns};
    AXIA_TRY(timed_pcg<double>(ctx, P, lanes, info));
    AXIA_TRY(read_out(ctx, &o));
    info->iters = o.iters;
    info->outer_iters = 1;
    info->residual = o.residual;
    info->bnorm = o.bnorm;
    if (o.status != AXIA_OK) {
      if (o.status == AXIA_ERR_NOT_CONVERGED)
        return set_error(ctx, o.status, "CG did not converge (residual " + std::to_string(o.residual) + " after " +
                                            std::to_string(o.iters) + " iterations)");
      if (o.status == AXIA_ERR_ZERO_PIVOT) return set_error(ctx, o.status, "CG: zero pivot, matrix not positive definite");
      return set_error(ctx, o.status, "CG: non-finite iterate");
    }
    return AXIA_OK;
  }
  // mixed: FP64 iterative refinement around an FP32 PCG on K32
  const int tb = 256, gb = ctx->sm_count * 8;
  AXIA_CUDA(ctx, cudaMemsetAsync(ctx->d_x, 0, n * sizeof(double), ctx->stream));
  AXIA_CUDA(ctx, cudaMemcpyAsync(ctx->d_r, ctx->d_b, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  std::vector<double> hb(1);
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
                     ctx->d_p32, ctx->d_q32, ctx->d_partials, ctx->d_bar, ctx->d_status, (PcgOut*)ctx->d_out, itol,
                     max_iter, limit_ns};
    AXIA_TRY(timed_pcg<float>(ctx, P, lanes, info));
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
    ctx->partial_slots = (size_t)N_SLOTS * 16 * 1024;
    AXIA_TRY(dev_alloc(ctx, &ctx->d_partials, ctx->partial_slots));
  }
  if (!ctx->d_bar) AXIA_TRY(dev_alloc(ctx, &ctx->d_bar, 1));
  if (!ctx->d_out) {
    PcgOut* o = nullptr;
    AXIA_TRY(dev_alloc(ctx, &o, 1));
    ctx->d_out = o;
  }
  return AXIA_OK;
}
