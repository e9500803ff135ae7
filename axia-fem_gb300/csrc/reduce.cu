// reduce.cu -- DofMap::reduce and reconstruct on the device, for models with
// multi-point constraints (the MPC path of solve_linear,
// solver/src/analysis.rs:1018-1025).
//
// DofMap::reduce (solver/src/constraint.rs:138-172) maps full-DOF triplets
// (i, j, v) to (a, b, v * t_ia * t_jb) for every pair of T entries of rows i
// and j, in triplet order, and builds rhs[a] from the load (rows ascending,
// T order) and then from -v * t_ia * u0_j per triplet (triplet order).  Here
// each source item (a triplet, or a load entry) gets its output count, a scan
// gives every item its output range, and one thread per item writes its
// outputs in the reference's order; the reduced triplets then go through the
// device csr_from_triplets (stable sort, in-order run sums), and the rhs
// contributions through the same stable sort by row with in-order sums, so
// K_ff and rhs equal the reference's bit for bit.  reconstruct
// (constraint.rs:207-217): u_d = u0_d + sum_k t_dk x_k in T order, one thread
// per DOF.
#include <algorithm>
#include <cmath>
#include <vector>

#include "solver.cuh"

int64_t dofmap_n_full(const axia_dofmap* m);
const int64_t* dofmap_t_ptr(const axia_dofmap* m);
const int64_t* dofmap_t_col(const axia_dofmap* m);
const double* dofmap_t_val(const axia_dofmap* m);
const double* dofmap_u0(const axia_dofmap* m);
int64_t dofmap_t_nnz(const axia_dofmap* m);

namespace {

// the reference skips a triplet only for an index past the end or an exact
// zero (a NaN passes and is dropped later by csr_from_triplets)
__device__ __forceinline__ bool trip_ok(int64_t i, int64_t j, double v, int64_t n_full) {
  return i >= 0 && j >= 0 && i < n_full && j < n_full && !(fabs(v) == 0.0);
}

// per triplet: reduced triplets it produces, and rhs terms it produces
__global__ void k_reduce_counts(int64_t nt, int64_t n_full, const int64_t* __restrict__ ti,
                                const int64_t* __restrict__ tj, const double* __restrict__ tv,
                                const int64_t* __restrict__ t_ptr, const double* __restrict__ u0,
                                int64_t* __restrict__ cnt_ff, int64_t* __restrict__ cnt_rhs, DevStatus* st) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nt; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = ti[k], j = tj[k];
    const double v = tv[k];
    if (i < 0 || j < 0) record_error(st, k, AXIA_ERR_INVALID_ARG);
    int64_t cf = 0, cr = 0;
    if (trip_ok(i, j, v, n_full)) {
      const int64_t li = t_ptr[i + 1] - t_ptr[i], lj = t_ptr[j + 1] - t_ptr[j];
      cf = li * lj;
      cr = fabs(u0[j]) > 0.0 ? li : 0;
    }
    cnt_ff[k] = cf;
    cnt_rhs[k] = cr;
  }
}

// per load entry: rhs terms it produces
__global__ void k_load_counts(int64_t n_full, const double* __restrict__ f, const int64_t* __restrict__ t_ptr,
                              int64_t* __restrict__ cnt) {
  for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < n_full; d += (int64_t)gridDim.x * blockDim.x)
    cnt[d] = fabs(f[d]) == 0.0 ? 0 : t_ptr[d + 1] - t_ptr[d];
}

// reduced triplets: key a * n_ind + b (sentinel n_ind^2 for a zero product), value v t_ia t_jb
__global__ void k_reduce_fill(int64_t nt, int64_t n_full, int64_t n_ind, const int64_t* __restrict__ ti,
                              const int64_t* __restrict__ tj, const double* __restrict__ tv,
                              const int64_t* __restrict__ t_ptr, const int64_t* __restrict__ t_col,
                              const double* __restrict__ t_val, const double* __restrict__ u0,
                              const int64_t* __restrict__ off_ff, const int64_t* __restrict__ off_rhs,
                              uint64_t* __restrict__ key_ff, double* __restrict__ val_ff,
                              uint64_t* __restrict__ key_rhs, double* __restrict__ val_rhs,
                              unsigned long long* __restrict__ n_valid) {
  const uint64_t sentinel = (uint64_t)n_ind * (uint64_t)n_ind;
  unsigned long long valid = 0;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nt; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = ti[k], j = tj[k];
    const double v = tv[k];
    if (!trip_ok(i, j, v, n_full)) continue;
    const double u0j = u0[j];
    int64_t pf = off_ff[k], pr = off_rhs[k];
    for (int64_t qa = t_ptr[i]; qa < t_ptr[i + 1]; ++qa) {
      const int64_t a = t_col[qa];
      const double vta = v * t_val[qa];
      if (fabs(u0j) > 0.0) {
        key_rhs[pr] = (uint64_t)a;
        val_rhs[pr] = -(vta * u0j);
        ++pr;
      }
      for (int64_t qb = t_ptr[j]; qb < t_ptr[j + 1]; ++qb) {
        const double w = vta * t_val[qb];
        const bool keep = fabs(w) > 0.0;
        key_ff[pf] = keep ? (uint64_t)a * (uint64_t)n_ind + (uint64_t)t_col[qb] : sentinel;
        val_ff[pf] = w;
        valid += keep ? 1ull : 0ull;
        ++pf;
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) valid += __shfl_down_sync(0xffffffffu, valid, o);
  if ((threadIdx.x & 31) == 0 && valid) atomicAdd(n_valid, valid);
}

__global__ void k_load_fill(int64_t n_full, const double* __restrict__ f, const int64_t* __restrict__ t_ptr,
                            const int64_t* __restrict__ t_col, const double* __restrict__ t_val,
                            const int64_t* __restrict__ off, uint64_t* __restrict__ key, double* __restrict__ val) {
  for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < n_full; d += (int64_t)gridDim.x * blockDim.x) {
    const double fd = f[d];
    if (fabs(fd) == 0.0) continue;
    int64_t p = off[d];
    for (int64_t q = t_ptr[d]; q < t_ptr[d + 1]; ++q, ++p) {
      key[p] = (uint64_t)t_col[q];
      val[p] = t_val[q] * fd;
    }
  }
}

__global__ void k_reconstruct_t(int64_t n_full, const int64_t* __restrict__ t_ptr, const int64_t* __restrict__ t_col,
                                const double* __restrict__ t_val, const double* __restrict__ u0,
                                const double* __restrict__ x, double* __restrict__ u) {
  for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < n_full; d += (int64_t)gridDim.x * blockDim.x) {
    double v = u0[d];
    for (int64_t q = t_ptr[d]; q < t_ptr[d + 1]; ++q) v += t_val[q] * x[t_col[q]];
    u[d] = v;
  }
}

unsigned grid_of(const axia_ctx* ctx, int64_t n) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->sm_count * 16));
}

}  // namespace


// K_ff = T^T K T in the context's raw CSR and rhs on the device.
int reduce_system(axia_ctx* ctx, const axia_dofmap* map, int64_t nt, const int64_t* h_i, const int64_t* h_j,
                  const double* h_v, const double* h_f, bool fp32, ReducedSystem* S) {
  S->n_full = dofmap_n_full(map);
  S->n_ind = axia_dofmap_n_ind(map);
  const int64_t nf = S->n_full, ni = S->n_ind, tn = dofmap_t_nnz(map);
  AXIA_TRY(dev_alloc(ctx, &S->t_ptr, (size_t)nf + 1));
  AXIA_TRY(dev_alloc(ctx, &S->t_col, (size_t)std::max<int64_t>(tn, 1)));
  AXIA_TRY(dev_alloc(ctx, &S->t_val, (size_t)std::max<int64_t>(tn, 1)));
  AXIA_TRY(dev_alloc(ctx, &S->u0, (size_t)nf));
  AXIA_TRY(dev_alloc(ctx, &S->rhs, (size_t)std::max<int64_t>(ni, 1)));
  cudaStream_t s = ctx->stream;
  AXIA_CUDA(ctx, cudaMemcpyAsync(S->t_ptr, dofmap_t_ptr(map), (nf + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, s));
  if (tn > 0) {
    AXIA_CUDA(ctx, cudaMemcpyAsync(S->t_col, dofmap_t_col(map), tn * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    AXIA_CUDA(ctx, cudaMemcpyAsync(S->t_val, dofmap_t_val(map), tn * sizeof(double), cudaMemcpyHostToDevice, s));
  }
  AXIA_CUDA(ctx, cudaMemcpyAsync(S->u0, dofmap_u0(map), nf * sizeof(double), cudaMemcpyHostToDevice, s));
  if (ni == 0) return AXIA_OK;
  // sources
  int64_t *di = nullptr, *dj = nullptr, *cnt = nullptr, *off = nullptr;
  double *dv = nullptr, *df = nullptr, *val_ff = nullptr, *val_rhs = nullptr;
  uint64_t *key_ff = nullptr, *key_rhs = nullptr;
  unsigned long long* dcount = nullptr;
  Runs Rk, Rr;
  int st = AXIA_OK;
  auto done = [&](int code) {
    cudaStreamSynchronize(ctx->stream);  // the temporaries return to the pool idle
    dev_release(ctx, di);
    dev_release(ctx, dj);
    dev_release(ctx, dv);
    dev_release(ctx, df);
    dev_release(ctx, cnt);
    dev_release(ctx, off);
    dev_release(ctx, val_ff);
    dev_release(ctx, val_rhs);
    dev_release(ctx, key_ff);
    dev_release(ctx, key_rhs);
    dev_release(ctx, dcount);
    Rk.release();
    Rr.release();
    return code;
  };
  const size_t m = (size_t)std::max<int64_t>(nt, 1);
  // counts: [0, nt) reduced triplets of each triplet; rhs items: [0, nf) load, [nf, nf + nt) triplets
  if ((st = dev_alloc(ctx, &di, m)) || (st = dev_alloc(ctx, &dj, m)) || (st = dev_alloc(ctx, &dv, m)) ||
      (st = dev_alloc(ctx, &df, (size_t)nf)) || (st = dev_alloc(ctx, &cnt, (size_t)(nt + nf + nt + 1))) ||
      (st = dev_alloc(ctx, &off, (size_t)(nt + nf + nt + 1))) || (st = dev_alloc(ctx, &dcount, 1)))
    return done(st);
  if (nt > 0 && (cudaMemcpyAsync(di, h_i, nt * sizeof(int64_t), cudaMemcpyHostToDevice, s) != cudaSuccess ||
                 cudaMemcpyAsync(dj, h_j, nt * sizeof(int64_t), cudaMemcpyHostToDevice, s) != cudaSuccess ||
                 cudaMemcpyAsync(dv, h_v, nt * sizeof(double), cudaMemcpyHostToDevice, s) != cudaSuccess))
    return done(set_error(ctx, AXIA_ERR_CUDA, "reduce: triplet upload"));
  if (cudaMemcpyAsync(df, h_f, nf * sizeof(double), cudaMemcpyHostToDevice, s) != cudaSuccess)
    return done(set_error(ctx, AXIA_ERR_CUDA, "reduce: load upload"));
  int64_t* cnt_ff = cnt;            // [nt]
  int64_t* cnt_load = cnt + nt;     // [nf]   rhs items in the reference's order:
  int64_t* cnt_trhs = cnt + nt + nf;  // [nt] load entries first, then triplets
  if (nt > 0) {
    k_reduce_counts<<<grid_of(ctx, nt), 256, 0, s>>>(nt, nf, di, dj, dv, S->t_ptr, S->u0, cnt_ff, cnt_trhs,
                                                     ctx->d_status);
    ctx->launches++;
  }
  k_load_counts<<<grid_of(ctx, nf), 256, 0, s>>>(nf, df, S->t_ptr, cnt_load);
  ctx->launches++;
  if (cudaGetLastError() != cudaSuccess) return done(set_error(ctx, AXIA_ERR_CUDA, "reduce: count kernels"));
  {
    DevStatus hs;
    if ((st = read_dev_status(ctx, &hs))) return done(st);
    if (hs.first_error != ~0ull) {
      ctx->last_bad = (int64_t)(hs.first_error >> 8);
      return done(set_error(ctx, AXIA_ERR_INVALID_ARG,
                            "reduce: triplet " + std::to_string(ctx->last_bad) + " has a negative index"));
    }
  }
  int64_t n_ff = 0, n_rhs = 0;
  if (nt > 0 && (st = device_exclusive_scan(ctx, cnt_ff, off, nt, &n_ff))) return done(st);
  if ((st = device_exclusive_scan(ctx, cnt_load, off + nt, nf + nt, &n_rhs))) return done(st);
  const size_t mf = (size_t)std::max<int64_t>(n_ff, 1), mr = (size_t)std::max<int64_t>(n_rhs, 1);
  if ((st = dev_alloc(ctx, &key_ff, mf)) || (st = dev_alloc(ctx, &val_ff, mf)) || (st = dev_alloc(ctx, &key_rhs, mr)) ||
      (st = dev_alloc(ctx, &val_rhs, mr)))
    return done(st);
  cudaMemsetAsync(dcount, 0, sizeof(unsigned long long), s);
  k_load_fill<<<grid_of(ctx, nf), 256, 0, s>>>(nf, df, S->t_ptr, S->t_col, S->t_val, off + nt, key_rhs, val_rhs);
  ctx->launches++;
  if (nt > 0) {
    k_reduce_fill<<<grid_of(ctx, nt), 256, 0, s>>>(nt, nf, ni, di, dj, dv, S->t_ptr, S->t_col, S->t_val, S->u0, off,
                                                   off + nt + nf, key_ff, val_ff, key_rhs, val_rhs, dcount);
    ctx->launches++;
  }
  if (cudaGetLastError() != cudaSuccess) return done(set_error(ctx, AXIA_ERR_CUDA, "reduce: fill kernels"));
  unsigned long long nv = 0;  // ordered after the fill kernel on the context's (non-blocking) stream
  if (cudaMemcpyAsync(&nv, dcount, sizeof(nv), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return done(set_error(ctx, AXIA_ERR_CUDA, "reduce: count"));
  if ((st = sort_runs(ctx, key_ff, val_ff, n_ff, (int64_t)nv, key_bits((uint64_t)ni * (uint64_t)ni), &Rk)))
    return done(st);
  if ((st = csr_from_runs(ctx, ni, Rk, fp32))) return done(st);
  if ((st = sort_runs(ctx, key_rhs, val_rhs, n_rhs, n_rhs, key_bits((uint64_t)ni), &Rr))) return done(st);
  if ((st = vector_from_runs(ctx, ni, Rr, S->rhs))) return done(st);
  if (cudaStreamSynchronize(s) != cudaSuccess) return done(set_error(ctx, AXIA_ERR_CUDA, "reduce"));
  return done(AXIA_OK);
}

int reconstruct_system(axia_ctx* ctx, const ReducedSystem& S, const double* d_x, double* d_u) {
  k_reconstruct_t<<<grid_of(ctx, S.n_full), 256, 0, ctx->stream>>>(S.n_full, S.t_ptr, S.t_col, S.t_val, S.u0, d_x,
                                                                    d_u);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  return AXIA_OK;
}
