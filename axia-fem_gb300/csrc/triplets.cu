// triplets.cu -- K_ff from a caller's triplets or CSR, for the solve_kff entry.
//
// The reference's solve_kff (solver/src/linalg.rs:311) receives K_ff as
// triplets and first runs csr_from_triplets (linalg.rs:10-38): keep the
// entries with i < n, j < n and |v| > 0 (a NaN value is dropped too, as
// `v.abs() > 0.0` is false for it), stable-sort by (i, j), sum each run of
// equal (i, j) from 0.0 in input order, store full symmetric CSR.  Here the
// same steps run on the device: key = i*n + j (a sentinel n*n for dropped
// entries), a stable LSD radix sort of (key, value) pairs (CUB), run heads
// flagged and scanned, one thread per run summing it left to right (the same
// additions in the same order as the reference), row pointers from the run
// rows, and the Jacobi diagonal of Csr::diag (linalg.rs:52-63: first entry of
// the row whose column is the row) with pcg's guard (linalg.rs:218-219).
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <cmath>
#include <vector>

#include "solver.cuh"

namespace {

__global__ void k_trip_keys(int64_t nt, int64_t n, const int64_t* __restrict__ ti, const int64_t* __restrict__ tj,
                            const double* __restrict__ tv, uint64_t* __restrict__ key,
                            unsigned long long* __restrict__ n_valid, DevStatus* st) {
  const uint64_t sentinel = (uint64_t)n * (uint64_t)n;
  unsigned long long cnt = 0;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nt; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = ti[k], j = tj[k];
    if (i < 0 || j < 0) {
      record_error(st, k, AXIA_ERR_INVALID_ARG);
      key[k] = sentinel;
      continue;
    }
    const bool keep = i < n && j < n && fabs(tv[k]) > 0.0;
    key[k] = keep ? (uint64_t)i * (uint64_t)n + (uint64_t)j : sentinel;
    cnt += keep ? 1ull : 0ull;
  }
  // per-warp sum, one integer atomic per warp (order-independent)
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(n_valid, cnt);
}

__global__ void k_run_flags(int64_t nv, const uint64_t* __restrict__ key, int64_t* __restrict__ flag) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nv; k += (int64_t)gridDim.x * blockDim.x)
    flag[k] = (k == 0 || key[k] != key[k - 1]) ? 1 : 0;
}

__global__ void k_run_heads(int64_t nv, const uint64_t* __restrict__ key, const int64_t* __restrict__ pos,
                            int64_t* __restrict__ head) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nv; k += (int64_t)gridDim.x * blockDim.x)
    if (k == 0 || key[k] != key[k - 1]) head[pos[k]] = k;
}

// One thread per run: the duplicate sum in input order, the column, and the
// row pointers of the rows from the previous run's row (exclusive) to this one.
__global__ void k_run_sum(int64_t nnz, int64_t nv, int64_t n, const uint64_t* __restrict__ key,
                          const double* __restrict__ val, const int64_t* __restrict__ head,
                          int32_t* __restrict__ rowptr, int32_t* __restrict__ col, double* __restrict__ out,
                          float* __restrict__ out32) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nnz; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = head[r], e = r + 1 < nnz ? head[r + 1] : nv;
    double v = 0.0;
    for (int64_t q = s; q < e; ++q) v += val[q];
    const uint64_t k = key[s];
    const int64_t row = (int64_t)(k / (uint64_t)n);
    col[r] = (int32_t)(k % (uint64_t)n);
    out[r] = v;
    if (out32) out32[r] = (float)v;
    const int64_t prev = r > 0 ? (int64_t)(key[head[r - 1]] / (uint64_t)n) : -1;
    for (int64_t i = prev + 1; i <= row; ++i) rowptr[i] = (int32_t)r;
    if (r == nnz - 1)
      for (int64_t i = row + 1; i <= n; ++i) rowptr[i] = (int32_t)nnz;
  }
}

// One thread per run: out[key] = run values summed from 0.0 in order.
__global__ void k_run_sum_vector(int64_t n_runs, int64_t nv, const uint64_t* __restrict__ key,
                                 const double* __restrict__ val, const int64_t* __restrict__ head,
                                 double* __restrict__ out) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n_runs; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = head[r], e = r + 1 < n_runs ? head[r + 1] : nv;
    double v = 0.0;
    for (int64_t q = s; q < e; ++q) v += val[q];
    out[key[s]] = v;
  }
}

__global__ void k_csr_to_i32(int64_t n, int64_t nnz, const int64_t* __restrict__ indptr,
                             const int64_t* __restrict__ indices, int32_t* __restrict__ rowptr,
                             int32_t* __restrict__ col, DevStatus* st) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nnz + n + 1;
       t += (int64_t)gridDim.x * blockDim.x) {
    if (t < nnz) {
      const int64_t c = indices[t];
      if (c < 0 || c >= n) {
        record_error(st, t, AXIA_ERR_INVALID_ARG);
        col[t] = 0;
      } else {
        col[t] = (int32_t)c;
      }
    } else {
      rowptr[t - nnz] = (int32_t)indptr[t - nnz];
    }
  }
}

__global__ void k_to_f32_values(int64_t n, const double* __restrict__ in, float* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (float)in[i];
}

__global__ void k_raw_diag(int64_t n, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                           const double* __restrict__ val, double* __restrict__ diag, double* __restrict__ dinv,
                           float* __restrict__ dinv32) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double d = 0.0;
    for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
      if (col[k] == i) {
        d = val[k];
        break;
      }
    diag[i] = d;
    const double di = fabs(d) > 1e-30 ? 1.0 / d : 1.0;
    dinv[i] = di;
    if (dinv32) dinv32[i] = (float)di;
  }
}

unsigned grid_for(const axia_ctx* ctx, int64_t n) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->sm_count * 16));
}

// CSR arrays of the raw system: rowptr, col, val (+ val32), diag, dinv (+ dinv32)
int alloc_raw(axia_ctx* ctx, int64_t n, int64_t nnz, bool fp32) {
  AXIA_TRY(dev_alloc(ctx, &ctx->d_rowptr, (size_t)n + 1));
  AXIA_TRY(dev_alloc(ctx, &ctx->d_col, (size_t)std::max<int64_t>(nnz, 1)));
  AXIA_TRY(dev_alloc(ctx, &ctx->d_val, (size_t)std::max<int64_t>(nnz, 1)));
  if (fp32) AXIA_TRY(dev_alloc(ctx, &ctx->d_val32, (size_t)std::max<int64_t>(nnz, 1)));
  AXIA_TRY(dev_alloc(ctx, &ctx->d_diag, (size_t)n));
  AXIA_TRY(dev_alloc(ctx, &ctx->d_dinv, (size_t)n));
  if (fp32) AXIA_TRY(dev_alloc(ctx, &ctx->d_dinv32, (size_t)n));
  return AXIA_OK;
}

int finish_raw(axia_ctx* ctx, int64_t n, int64_t nnz, bool fp32) {
  k_raw_diag<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(n, ctx->d_rowptr, ctx->d_col, ctx->d_val, ctx->d_diag,
                                                        ctx->d_dinv, fp32 ? ctx->d_dinv32 : nullptr);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  ctx->n_free = ctx->ndof = n;
  ctx->nnz = nnz;
  ctx->assembled = ctx->have_csr64 = true;
  ctx->have32 = fp32;
  return AXIA_OK;
}

int check_status(axia_ctx* ctx, const char* what) {
  DevStatus hs;
  AXIA_TRY(read_dev_status(ctx, &hs));
  if (hs.first_error != ~0ull) {
    ctx->last_bad = (int64_t)(hs.first_error >> 8);
    return set_error(ctx, (int)(hs.first_error & 0xff),
                     std::string(what) + ": entry " + std::to_string(ctx->last_bad) + " has an index out of range");
  }
  return AXIA_OK;
}

}  // namespace

// Stable radix sort of (key, value) over end_bit key bits and the runs of
// equal keys among the first nv sorted entries (the entries to drop carry a
// sentinel key above every valid one, so they sort last).  dk / dv are the
// unsorted inputs (nt entries) and are left untouched.
int sort_runs(axia_ctx* ctx, const uint64_t* dk, const double* dv, int64_t nt, int64_t nv, int end_bit, Runs* out) {
  *out = Runs{};
  out->nv = nv;
  if (nt <= 0 || nv <= 0) return AXIA_OK;
  const size_t m = (size_t)nt;
  AXIA_TRY(dev_alloc(ctx, &out->key, m));
  AXIA_TRY(dev_alloc(ctx, &out->val, m));
  size_t temp_bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, temp_bytes, dk, out->key, dv, out->val, nt, 0, end_bit, ctx->stream);
  void* temp = nullptr;
  if (cudaMalloc(&temp, std::max<size_t>(temp_bytes, 1)) != cudaSuccess)
    return set_error(ctx, AXIA_ERR_OOM, "sort workspace");
  const cudaError_t e = cub::DeviceRadixSort::SortPairs(temp, temp_bytes, dk, out->key, dv, out->val, nt, 0, end_bit,
                                                        ctx->stream);
  cudaStreamSynchronize(ctx->stream);  // the sort has finished with its workspace
  cudaFree(temp);
  if (e != cudaSuccess) return set_error(ctx, AXIA_ERR_CUDA, "radix sort");
  ctx->launches++;
  int64_t *flag = nullptr, *pos = nullptr;
  AXIA_TRY(dev_alloc(ctx, &flag, (size_t)nv));
  int st = dev_alloc(ctx, &pos, (size_t)nv);
  if (st == AXIA_OK) {
    k_run_flags<<<grid_for(ctx, nv), 256, 0, ctx->stream>>>(nv, out->key, flag);
    ctx->launches++;
    st = device_exclusive_scan(ctx, flag, pos, nv, &out->n_runs);
  }
  if (st == AXIA_OK && out->n_runs > 0) st = dev_alloc(ctx, &out->head, (size_t)out->n_runs);
  if (st == AXIA_OK && out->n_runs > 0) {
    k_run_heads<<<grid_for(ctx, nv), 256, 0, ctx->stream>>>(nv, out->key, pos, out->head);
    ctx->launches++;
  }
  cudaStreamSynchronize(ctx->stream);  // the temporaries return to the pool idle
  dev_release(ctx, flag);
  dev_release(ctx, pos);
  if (st == AXIA_OK && cudaGetLastError() != cudaSuccess) st = set_error(ctx, AXIA_ERR_CUDA, "run kernels");
  return st;
}

int key_bits(uint64_t max_key) {
  int b = 1;
  while (b < 64 && (max_key >> b) != 0) ++b;
  return b;
}

// The context's raw CSR from sorted runs of keys i*n + j.
int csr_from_runs(axia_ctx* ctx, int64_t n, const Runs& R, bool fp32) {
  const int64_t nnz = R.n_runs;
  if (nnz >= (int64_t)INT32_MAX) return set_error(ctx, AXIA_ERR_TOO_LARGE, "K_ff: nnz exceeds int32");
  AXIA_TRY(alloc_raw(ctx, n, nnz, fp32));
  if (nnz > 0) {
    k_run_sum<<<grid_for(ctx, nnz), 256, 0, ctx->stream>>>(nnz, R.nv, n, R.key, R.val, R.head, ctx->d_rowptr,
                                                           ctx->d_col, ctx->d_val, fp32 ? ctx->d_val32 : nullptr);
    ctx->launches++;
  } else {
    cudaMemsetAsync(ctx->d_rowptr, 0, (n + 1) * sizeof(int32_t), ctx->stream);
  }
  if (cudaGetLastError() != cudaSuccess) return set_error(ctx, AXIA_ERR_CUDA, "CSR kernels");
  return finish_raw(ctx, n, nnz, fp32);
}

// out[key] = the run's values summed from 0.0 in order; keys without a run get 0.
int vector_from_runs(axia_ctx* ctx, int64_t n, const Runs& R, double* d_out) {
  AXIA_CUDA(ctx, cudaMemsetAsync(d_out, 0, std::max<int64_t>(n, 1) * sizeof(double), ctx->stream));
  if (R.n_runs > 0) {
    k_run_sum_vector<<<grid_for(ctx, R.n_runs), 256, 0, ctx->stream>>>(R.n_runs, R.nv, R.key, R.val, R.head, d_out);
    ctx->launches++;
  }
  AXIA_CUDA(ctx, cudaGetLastError());
  return AXIA_OK;
}

// K_ff from triplets (host arrays) into the context's CSR (int32 indices).
int raw_system_from_triplets(axia_ctx* ctx, int64_t n, int64_t nt, const int64_t* h_i, const int64_t* h_j,
                             const double* h_v, bool fp32) {
  if (n <= 0 || n >= (int64_t)INT32_MAX || nt < 0) return set_error(ctx, AXIA_ERR_INVALID_ARG, "solve_kff: bad n or triplet count");
  AXIA_TRY(reset_dev_status(ctx));
  int64_t *di = nullptr, *dj = nullptr;
  double* dv = nullptr;
  uint64_t* dk = nullptr;
  unsigned long long* dcount = nullptr;
  Runs R;
  int st = AXIA_OK;
  auto done = [&](int code) {
    cudaStreamSynchronize(ctx->stream);  // the temporaries return to the pool idle
    dev_release(ctx, di);
    dev_release(ctx, dj);
    dev_release(ctx, dv);
    dev_release(ctx, dk);
    dev_release(ctx, dcount);
    R.release();
    return code;
  };
  const size_t m = (size_t)std::max<int64_t>(nt, 1);
  if ((st = dev_alloc(ctx, &di, m)) || (st = dev_alloc(ctx, &dj, m)) || (st = dev_alloc(ctx, &dv, m)) ||
      (st = dev_alloc(ctx, &dk, m)) || (st = dev_alloc(ctx, &dcount, 1)))
    return done(st);
  if (nt > 0) {
    if (cudaMemcpyAsync(di, h_i, nt * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
        cudaMemcpyAsync(dj, h_j, nt * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
        cudaMemcpyAsync(dv, h_v, nt * sizeof(double), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
      return done(set_error(ctx, AXIA_ERR_CUDA, "solve_kff: triplet upload"));
  }
  cudaMemsetAsync(dcount, 0, sizeof(unsigned long long), ctx->stream);
  if (nt > 0) {
    k_trip_keys<<<grid_for(ctx, nt), 256, 0, ctx->stream>>>(nt, n, di, dj, dv, dk, dcount, ctx->d_status);
    ctx->launches++;
  }
  if (cudaGetLastError() != cudaSuccess) return done(set_error(ctx, AXIA_ERR_CUDA, "solve_kff: key kernel"));
  if ((st = check_status(ctx, "solve_kff triplets"))) return done(st);
  unsigned long long nv = 0;  // ordered after the key kernel on the context's (non-blocking) stream
  if (cudaMemcpyAsync(&nv, dcount, sizeof(nv), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
      cudaStreamSynchronize(ctx->stream) != cudaSuccess)
    return done(set_error(ctx, AXIA_ERR_CUDA, "solve_kff: count"));
  if ((st = sort_runs(ctx, dk, dv, nt, (int64_t)nv, key_bits((uint64_t)n * (uint64_t)n), &R))) return done(st);
  if ((st = csr_from_runs(ctx, n, R, fp32))) return done(st);
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess)
    return done(set_error(ctx, AXIA_ERR_CUDA, "solve_kff: CSR build"));
  return done(AXIA_OK);
}

// K_ff from a CSR the caller built (int64 indptr / indices, as the reference's Csr).
int raw_system_from_csr(axia_ctx* ctx, int64_t n, const int64_t* h_indptr, const int64_t* h_indices,
                        const double* h_data, bool fp32) {
  if (n <= 0 || n >= (int64_t)INT32_MAX) return set_error(ctx, AXIA_ERR_INVALID_ARG, "solve_csr: bad n");
  if (h_indptr[0] != 0) return set_error(ctx, AXIA_ERR_INVALID_ARG, "solve_csr: indptr[0] != 0");
  for (int64_t i = 0; i < n; ++i)
    if (h_indptr[i + 1] < h_indptr[i]) {
      ctx->last_bad = i;
      return set_error(ctx, AXIA_ERR_INVALID_ARG, "solve_csr: indptr decreases at row " + std::to_string(i));
    }
  const int64_t nnz = h_indptr[n];
  if (nnz >= (int64_t)INT32_MAX) return set_error(ctx, AXIA_ERR_TOO_LARGE, "solve_csr: nnz exceeds int32");
  AXIA_TRY(reset_dev_status(ctx));
  AXIA_TRY(alloc_raw(ctx, n, nnz, fp32));
  int64_t *dp = nullptr, *dc = nullptr;
  AXIA_TRY(dev_alloc(ctx, &dp, (size_t)n + 1));
  int st = dev_alloc(ctx, &dc, (size_t)std::max<int64_t>(nnz, 1));
  if (st == AXIA_OK) {
    cudaMemcpyAsync(dp, h_indptr, (n + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream);
    if (nnz > 0) {
      cudaMemcpyAsync(dc, h_indices, nnz * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream);
      cudaMemcpyAsync(ctx->d_val, h_data, nnz * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    }
    k_csr_to_i32<<<grid_for(ctx, nnz + n + 1), 256, 0, ctx->stream>>>(n, nnz, dp, dc, ctx->d_rowptr, ctx->d_col,
                                                                       ctx->d_status);
    ctx->launches++;
    if (cudaGetLastError() != cudaSuccess) st = set_error(ctx, AXIA_ERR_CUDA, "solve_csr: conversion kernel");
  }
  if (st == AXIA_OK) st = check_status(ctx, "solve_csr column");
  if (st == AXIA_OK && fp32 && nnz > 0) {
    k_to_f32_values<<<grid_for(ctx, nnz), 256, 0, ctx->stream>>>(nnz, ctx->d_val, ctx->d_val32);
    ctx->launches++;
  }
  if (st == AXIA_OK) st = finish_raw(ctx, n, nnz, fp32);
  cudaStreamSynchronize(ctx->stream);
  dev_release(ctx, dp);
  dev_release(ctx, dc);
  return st;
}
