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

// K_ff from triplets (host arrays) into the context's CSR (int32 indices).
int raw_system_from_triplets(axia_ctx* ctx, int64_t n, int64_t nt, const int64_t* h_i, const int64_t* h_j,
                             const double* h_v, bool fp32) {
  if (n <= 0 || n >= (int64_t)INT32_MAX || nt < 0) return set_error(ctx, AXIA_ERR_INVALID_ARG, "solve_kff: bad n or triplet count");
  AXIA_TRY(reset_dev_status(ctx));
  int64_t *di = nullptr, *dj = nullptr;
  double *dv = nullptr, *dv_sorted = nullptr;
  uint64_t *dk = nullptr, *dk_sorted = nullptr;
  unsigned long long* dcount = nullptr;
  int64_t *flag = nullptr, *pos = nullptr, *head = nullptr;
  void* temp = nullptr;
  int st = AXIA_OK;
  auto fail = [&](int code) {
    dev_free(di);
    dev_free(dj);
    dev_free(dv);
    dev_free(dv_sorted);
    dev_free(dk);
    dev_free(dk_sorted);
    dev_free(dcount);
    dev_free(flag);
    dev_free(pos);
    dev_free(head);
    if (temp) cudaFree(temp);
    return code;
  };
  const size_t m = (size_t)std::max<int64_t>(nt, 1);
  if ((st = dev_alloc(ctx, &di, m)) || (st = dev_alloc(ctx, &dj, m)) || (st = dev_alloc(ctx, &dv, m)) ||
      (st = dev_alloc(ctx, &dk, m)) || (st = dev_alloc(ctx, &dcount, 1)))
    return fail(st);
  if (nt > 0) {
    if (cudaMemcpyAsync(di, h_i, nt * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
        cudaMemcpyAsync(dj, h_j, nt * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
        cudaMemcpyAsync(dv, h_v, nt * sizeof(double), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
      return fail(set_error(ctx, AXIA_ERR_CUDA, "solve_kff: triplet upload"));
  }
  cudaMemsetAsync(dcount, 0, sizeof(unsigned long long), ctx->stream);
  if (nt > 0) {
    k_trip_keys<<<grid_for(ctx, nt), 256, 0, ctx->stream>>>(nt, n, di, dj, dv, dk, dcount, ctx->d_status);
    ctx->launches++;
  }
  if (cudaGetLastError() != cudaSuccess) return fail(set_error(ctx, AXIA_ERR_CUDA, "solve_kff: key kernel"));
  if ((st = check_status(ctx, "solve_kff triplets"))) return fail(st);
  dev_free(di);
  dev_free(dj);
  unsigned long long nv_h = 0;
  if (cudaMemcpy(&nv_h, dcount, sizeof(nv_h), cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail(set_error(ctx, AXIA_ERR_CUDA, "solve_kff: count"));
  const int64_t nv = (int64_t)nv_h;
  // stable radix sort of (key, value) over the bits that n*n needs
  const uint64_t sentinel = (uint64_t)n * (uint64_t)n;
  int end_bit = 1;
  while (end_bit < 64 && (sentinel >> end_bit) != 0) ++end_bit;
  if (nt > 0) {
    if ((st = dev_alloc(ctx, &dk_sorted, m)) || (st = dev_alloc(ctx, &dv_sorted, m))) return fail(st);
    size_t temp_bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, temp_bytes, dk, dk_sorted, dv, dv_sorted, nt, 0, end_bit, ctx->stream);
    if (cudaMalloc(&temp, std::max<size_t>(temp_bytes, 1)) != cudaSuccess)
      return fail(set_error(ctx, AXIA_ERR_OOM, "solve_kff: sort workspace"));
    if (cub::DeviceRadixSort::SortPairs(temp, temp_bytes, dk, dk_sorted, dv, dv_sorted, nt, 0, end_bit,
                                        ctx->stream) != cudaSuccess)
      return fail(set_error(ctx, AXIA_ERR_CUDA, "solve_kff: radix sort"));
    ctx->launches++;
    cudaFree(temp);
    temp = nullptr;
    dev_free(dk);
    dev_free(dv);
  }
  // run heads -> unique (i, j) entries
  int64_t nnz = 0;
  if (nv > 0) {
    if ((st = dev_alloc(ctx, &flag, (size_t)nv)) || (st = dev_alloc(ctx, &pos, (size_t)nv))) return fail(st);
    k_run_flags<<<grid_for(ctx, nv), 256, 0, ctx->stream>>>(nv, dk_sorted, flag);
    ctx->launches++;
    if ((st = device_exclusive_scan(ctx, flag, pos, nv, &nnz))) return fail(st);
  }
  if (nnz >= (int64_t)INT32_MAX) return fail(set_error(ctx, AXIA_ERR_TOO_LARGE, "solve_kff: nnz exceeds int32"));
  if ((st = alloc_raw(ctx, n, nnz, fp32))) return fail(st);
  if (nnz > 0) {
    if ((st = dev_alloc(ctx, &head, (size_t)nnz))) return fail(st);
    k_run_heads<<<grid_for(ctx, nv), 256, 0, ctx->stream>>>(nv, dk_sorted, pos, head);
    k_run_sum<<<grid_for(ctx, nnz), 256, 0, ctx->stream>>>(nnz, nv, n, dk_sorted, dv_sorted, head, ctx->d_rowptr,
                                                           ctx->d_col, ctx->d_val, fp32 ? ctx->d_val32 : nullptr);
    ctx->launches += 2;
  } else {
    cudaMemsetAsync(ctx->d_rowptr, 0, (n + 1) * sizeof(int32_t), ctx->stream);
  }
  if (cudaGetLastError() != cudaSuccess) return fail(set_error(ctx, AXIA_ERR_CUDA, "solve_kff: CSR kernels"));
  if ((st = finish_raw(ctx, n, nnz, fp32))) return fail(st);
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess)
    return fail(set_error(ctx, AXIA_ERR_CUDA, "solve_kff: CSR build"));
  return fail(AXIA_OK);
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
  dev_free(dp);
  dev_free(dc);
  return st;
}
