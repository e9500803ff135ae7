// util.cu -- device exclusive scan, status word, error strings.
#include <algorithm>

#include "common.cuh"

int set_error(axia_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->last_error = msg;
  return code;
}

int read_dev_status(axia_ctx* ctx, DevStatus* st_host) {
  AXIA_CUDA(ctx, cudaMemcpyAsync(st_host, ctx->d_status, sizeof(DevStatus), cudaMemcpyDeviceToHost, ctx->stream));
  AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return AXIA_OK;
}

int reset_dev_status(axia_ctx* ctx) {
  DevStatus clean;
  clean.first_error = ~0ull;
  clean.timeout = 0;
  clean.pad = 0;
  AXIA_CUDA(ctx, cudaMemcpyAsync(ctx->d_status, &clean, sizeof(DevStatus), cudaMemcpyHostToDevice, ctx->stream));
  return AXIA_OK;
}

__global__ void k_first_nonfinite(int64_t n, const double* v, unsigned long long* first) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (!isfinite(v[i])) atomicMin(first, (unsigned long long)i);
}

int device_first_nonfinite(axia_ctx* ctx, const double* d_v, int64_t n, int64_t* first) {
  *first = -1;
  if (n <= 0) return AXIA_OK;
  if (!ctx->d_first_bad) AXIA_TRY(dev_alloc(ctx, &ctx->d_first_bad, 1));
  AXIA_CUDA(ctx, cudaMemsetAsync(ctx->d_first_bad, 0xff, sizeof(unsigned long long), ctx->stream));
  const int64_t want = (n + 255) / 256, cap = (int64_t)ctx->sm_count * 8;
  k_first_nonfinite<<<(unsigned)(want < cap ? want : cap), 256, 0, ctx->stream>>>(n, d_v, ctx->d_first_bad);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  unsigned long long h = ~0ull;
  AXIA_CUDA(ctx, cudaMemcpyAsync(&h, ctx->d_first_bad, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (h != ~0ull) *first = (int64_t)h;
  return AXIA_OK;
}

// ---------------------------------------------------------------------------
// Exclusive scan of int64 counts: block-local scan of SCAN_ITEMS per block,
// scan of the block totals (recursively), then add the block offsets.
// ---------------------------------------------------------------------------
constexpr int SCAN_THREADS = 512;
constexpr int SCAN_PER_THREAD = 8;
constexpr int SCAN_ITEMS = SCAN_THREADS * SCAN_PER_THREAD;

__global__ void __launch_bounds__(SCAN_THREADS)
k_scan_block(const int64_t* in, int64_t* out, int64_t n, int64_t* block_tot) {
  __shared__ int64_t s_warp[SCAN_THREADS / 32];
  const int64_t base = (int64_t)blockIdx.x * SCAN_ITEMS + (int64_t)threadIdx.x * SCAN_PER_THREAD;
  int64_t v[SCAN_PER_THREAD];
  int64_t sum = 0;
#pragma unroll
  for (int k = 0; k < SCAN_PER_THREAD; ++k) {
    int64_t i = base + k;
    v[k] = i < n ? in[i] : 0;
    sum += v[k];
  }
  // inclusive scan of per-thread sums within the warp
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t inc = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) s_warp[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    int64_t w = lane < SCAN_THREADS / 32 ? s_warp[lane] : 0;
    int64_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    if (lane < SCAN_THREADS / 32) s_warp[lane] = wi - w;  // exclusive warp offsets
    if (lane == SCAN_THREADS / 32 - 1 && block_tot) block_tot[blockIdx.x] = wi;
  }
  __syncthreads();
  int64_t run = s_warp[warp] + inc - sum;
#pragma unroll
  for (int k = 0; k < SCAN_PER_THREAD; ++k) {
    int64_t i = base + k;
    int64_t x = v[k];
    if (i < n) out[i] = run;
    run += x;
  }
}

__global__ void k_scan_add(int64_t* out, int64_t n, const int64_t* offs) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += offs[i / SCAN_ITEMS];
}

int device_exclusive_scan(axia_ctx* ctx, const int64_t* d_in, int64_t* d_out, int64_t n, int64_t* total) {
  if (n <= 0) {
    *total = 0;
    return AXIA_OK;
  }
  const int64_t nb = (n + SCAN_ITEMS - 1) / SCAN_ITEMS;
  int64_t* d_tot = nullptr;
  int64_t* d_tot_scan = nullptr;
  AXIA_TRY(dev_alloc(ctx, &d_tot, nb));
  AXIA_TRY(dev_alloc(ctx, &d_tot_scan, nb));
  // last input element (for the total), read before an in-place scan overwrites it
  int64_t last_in = 0;
  AXIA_CUDA(ctx, cudaMemcpyAsync(&last_in, d_in + (n - 1), sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
  AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  k_scan_block<<<(unsigned)nb, SCAN_THREADS, 0, ctx->stream>>>(d_in, d_out, n, d_tot);
  AXIA_CUDA(ctx, cudaGetLastError());
  if (nb > 1) {
    int64_t t2 = 0;
    AXIA_TRY(device_exclusive_scan(ctx, d_tot, d_tot_scan, nb, &t2));
    k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(d_out, n, d_tot_scan);
    AXIA_CUDA(ctx, cudaGetLastError());
  }
  int64_t last_out = 0;
  AXIA_CUDA(ctx, cudaMemcpyAsync(&last_out, d_out + (n - 1), sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
  AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  *total = last_out + last_in;
  dev_release(ctx, d_tot);
  dev_release(ctx, d_tot_scan);
  return AXIA_OK;
}

// ---------------------------------------------------------------------------
// FMA throughput probe: every thread runs NCH independent chains of
// a = fma(a, m, c) (2 flops each), the grid fills every SM; the rate is the
// flops over the kernel's CUDA-event time (best of three launches).  It gives
// the FP64 (and FP32) denominators of the element kernel's roofline.
// ---------------------------------------------------------------------------
template <typename T, int NCH>
__global__ void __launch_bounds__(256) k_fma_rate(int iters, T m, T c, T* sink) {
  T a[NCH];
#pragma unroll
  for (int k = 0; k < NCH; ++k) a[k] = T(threadIdx.x + k) * T(1e-3);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < NCH; ++k) a[k] = fma(a[k], m, c);
  }
  T s = T(0);
#pragma unroll
  for (int k = 0; k < NCH; ++k) s += a[k];
  if (s == T(-1.0)) sink[blockIdx.x] = s;  // never true for these inputs; keeps the chains live
}

template <typename T, int NCH>
static int fma_rate(axia_ctx* ctx, int iters, double* tflops) {
  auto kern = k_fma_rate<T, NCH>;
  int per_sm = 0;
  AXIA_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, 0));
  const int grid = std::max(1, per_sm) * ctx->sm_count;
  T* sink = nullptr;
  AXIA_TRY(dev_alloc(ctx, &sink, (size_t)grid));
  cudaEvent_t a, b;
  AXIA_CUDA(ctx, cudaEventCreate(&a));
  AXIA_CUDA(ctx, cudaEventCreate(&b));
  float best = 0.f;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(a, ctx->stream);
    kern<<<grid, 256, 0, ctx->stream>>>(iters, T(0.9999999), T(1e-7), sink);
    cudaEventRecord(b, ctx->stream);
    ctx->launches++;
    AXIA_CUDA(ctx, cudaEventSynchronize(b));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (rep > 0 && (best == 0.f || ms < best)) best = ms;  // the first launch warms up
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  dev_release(ctx, sink);
  AXIA_CUDA(ctx, cudaGetLastError());
  const double flops = 2.0 * NCH * (double)iters * (double)grid * 256.0;
  *tflops = flops / (best * 1e-3) / 1e12;
  return AXIA_OK;
}

extern "C" AXIA_API int32_t axia_gpu_fma_rate(axia_ctx* ctx, int32_t precision, double* tflops) {
  if (!ctx || !tflops) return AXIA_ERR_INVALID_ARG;
  AXIA_CUDA(ctx, cudaSetDevice(ctx->device));
  if (precision == AXIA_PREC_FP64) return fma_rate<double, 8>(ctx, 2048, tflops);
  return fma_rate<float, 16>(ctx, 16384, tflops);
}
