// common.cuh -- context, error plumbing and device utilities shared by the
// kernels of libaxia_gpu.so (GB300, sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/axia_gpu.h"

// ---------------------------------------------------------------------------
// Device-side status word.  Kernels never trap: they record the first error
// (lowest element / row index wins) and return.
// code in the low 8 bits, index in the upper 56 bits, so atomicMin picks the
// lowest index, as the reference's sequential element loop reports the first
// failing element (solver/src/analysis.rs:574-628).
// ---------------------------------------------------------------------------
struct DevStatus {
  unsigned long long first_error;  // (index << 8) | code, ~0ull when clean
  int timeout;                     // set by a wait that ran past its limit
  int pad;
};

__device__ __forceinline__ void record_error(DevStatus* st, long long index, int code) {
  unsigned long long key = ((unsigned long long)index << 8) | (unsigned long long)(code & 0xff);
  atomicMin(&st->first_error, key);
}

// Nanosecond clock used to bound every spin-wait.
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_gpu(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// s = 0 + p[0] + p[stride] + ... + p[(n-1) stride] in that order, read with
// ld.cg (values another block or warp wrote), eight loads in flight at a time.
template <typename T>
__device__ __forceinline__ T ldcg_sum(const T* p, size_t stride, int n) {
  T s = T(0);
  int k = 0;
  for (; k + 8 <= n; k += 8) {
    T v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = __ldcg(p + (size_t)(k + u) * stride);
#pragma unroll
    for (int u = 0; u < 8; ++u) s += v[u];
  }
  for (; k < n; ++k) s += __ldcg(p + (size_t)k * stride);
  return s;
}

// Grid-wide barrier for a cooperative (co-resident) launch: one 64-bit word,
// generation in the upper half, arrivals at the current barrier in the lower
// half (the host zeroes it before every launch).  An arrival is one atomic
// add; the last block stores (generation + 1) << 32, which releases the
// others and re-arms the count in one write (no block can arrive at the next
// barrier before that store).  The wait is bounded: after `limit_ns`, or once
// another block has recorded a timeout, the block records it and returns
// false; every caller then leaves its loop, so a stuck barrier ends all blocks.
struct GridBarrier {
  unsigned long long word;
  unsigned long long pad[15];  // one L2 line per barrier
};

__device__ __forceinline__ unsigned long long ld_acquire_gpu64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_gpu64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ unsigned long long ld_relaxed_gpu64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// Arrival of the calling block (one thread): its writes are released and the
// generation it waits past is returned; *last is set for the final arrival,
// which has then acquired every other block's writes.  The blocks of a group
// barrier (the CTAs of one system inside a multi-system launch, nblk <
// gridDim.x) first read the word once: measured on 64 meshes in one launch,
// the solve ran 22 % faster with that read, while a whole-grid barrier ran
// 0.4 % slower with it, so only group barriers take it.
__device__ __forceinline__ unsigned barrier_arrive(GridBarrier* bar, unsigned nblk, int* last) {
  if (nblk != gridDim.x) (void)ld_acquire_gpu64(&bar->word);
  __threadfence();
  const unsigned long long old = atomicAdd(&bar->word, 1ull);
  *last = (unsigned)(old & 0xffffffffull) == nblk - 1;
  if (*last) __threadfence();
  return (unsigned)(old >> 32);
}

__device__ __forceinline__ void barrier_release(GridBarrier* bar, unsigned g) {
  st_release_gpu64(&bar->word, (unsigned long long)(g + 1u) << 32);
}

// Bounded wait (one thread) until generation g has been released.  The polls
// are relaxed loads (an acquire load per poll costs the blocks that share the
// SM measurably: 1 % on the two-level CG); the fence after the loop that saw
// the release makes it an acquire.
__device__ __forceinline__ bool barrier_wait(GridBarrier* bar, DevStatus* st, unsigned long long limit_ns, unsigned g) {
  const unsigned long long t0 = global_ns();
  unsigned spins = 0;
  while ((unsigned)(ld_relaxed_gpu64(&bar->word) >> 32) == g) {
    if ((++spins & 63u) == 0) {
      if (*(volatile int*)&st->timeout) return false;
      if (global_ns() - t0 > limit_ns) {
        atomicExch(&st->timeout, 1);
        return false;
      }
    }
    if (spins > 128) __nanosleep(32);
  }
  __threadfence();
  return true;
}

// Barrier over a group of nblk co-resident blocks (the whole grid: nblk = gridDim.x).
__device__ __forceinline__ bool group_sync(GridBarrier* bar, DevStatus* st, unsigned long long limit_ns, unsigned nblk) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int last;
    const unsigned g = barrier_arrive(bar, nblk, &last);
    int ok = 1;
    if (last)
      barrier_release(bar, g);
    else
      ok = barrier_wait(bar, st, limit_ns, g);
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ bool grid_sync(GridBarrier* bar, DevStatus* st, unsigned long long limit_ns) {
  return group_sync(bar, st, limit_ns, gridDim.x);
}

// Grid-wide barrier that also reduces.  Every block has stored its partials of
// nv <= 4 values at partials[(slot0 + k) * nblk + rank]; the last block to
// arrive sums them with all its threads (one L2 round trip; thread t takes
// blocks t, t + blockDim.x, ..., then warps and the warp sums in order: a fixed
// order, so every run gives the same bits) and publishes totals[slot0 + k]
// before it releases the others.  Same bounded wait as grid_sync.  With res,
// thread 0 of every block copies the totals into shared memory and every
// thread gets them in res[0..nv) (one L2 read per block instead of one per
// warp on a single line); without, threads read totals[] with ld.cg.
constexpr int REDUCE_MAX_NV = 4;

// The last block's part of group_reduce_sync (every thread of the block calls
// it).  Not inlined: its registers stay out of the allocation of the CG loops
// that call the barrier.
static __device__ __noinline__ void reduce_partials_last_block(const double* partials, double* totals, double* s_tot,
                                                        int slot0, int nv, unsigned nblk) {
  __shared__ double s_sum[REDUCE_MAX_NV][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  double a[REDUCE_MAX_NV];
#pragma unroll
  for (int k = 0; k < REDUCE_MAX_NV; ++k) a[k] = 0.0;
  for (int j = threadIdx.x; j < (int)nblk; j += blockDim.x) {
    double v[REDUCE_MAX_NV];
#pragma unroll
    for (int k = 0; k < REDUCE_MAX_NV; ++k) v[k] = k < nv ? __ldcg(partials + (size_t)(slot0 + k) * nblk + j) : 0.0;
#pragma unroll
    for (int k = 0; k < REDUCE_MAX_NV; ++k) a[k] += v[k];
  }
#pragma unroll
  for (int k = 0; k < REDUCE_MAX_NV; ++k) {
    if (k < nv) {
      a[k] = warp_sum(a[k]);
      if (lane == 0) s_sum[k][warp] = a[k];
    }
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < REDUCE_MAX_NV; ++k) {
      if (k < nv) {
        double t = lane < nw ? s_sum[k][lane] : 0.0;
        t = warp_sum(t);
        if (lane == 0) {
          totals[slot0 + k] = t;
          s_tot[k] = t;
        }
      }
    }
  }
}

__device__ __forceinline__ bool group_reduce_sync(GridBarrier* bar, DevStatus* st, unsigned long long limit_ns,
                                                  const double* partials, double* totals, int slot0, int nv,
                                                  unsigned nblk, double* res = nullptr) {
  __shared__ int s_last, s_ok2;
  __shared__ unsigned s_gen;
  __shared__ double s_tot[REDUCE_MAX_NV];
  __syncthreads();
  if (threadIdx.x == 0) {
    int last;
    s_gen = barrier_arrive(bar, nblk, &last);
    s_last = last;
  }
  __syncthreads();
  int ok = 1;
  if (s_last) {
    reduce_partials_last_block(partials, totals, s_tot, slot0, nv, nblk);
    if (threadIdx.x == 0) {
      __threadfence();
      barrier_release(bar, s_gen);
    }
  } else if (threadIdx.x == 0) {
    ok = barrier_wait(bar, st, limit_ns, s_gen);
    if (ok && res)
      for (int k = 0; k < nv; ++k) s_tot[k] = __ldcg(totals + slot0 + k);
  }
  if (threadIdx.x == 0) s_ok2 = ok;
  __syncthreads();
  if (res)
    for (int k = 0; k < nv; ++k) res[k] = s_tot[k];
  return s_ok2 != 0;
}

__device__ __forceinline__ bool grid_reduce_sync(GridBarrier* bar, DevStatus* st, unsigned long long limit_ns,
                                                 const double* partials, double* totals, int slot0, int nv,
                                                 double* res = nullptr) {
  return group_reduce_sync(bar, st, limit_ns, partials, totals, slot0, nv, gridDim.x, res);
}

// Streaming (evict-first) loads for matrix data that is read once per sweep,
// so the vectors keep their L2 lines.
__device__ __forceinline__ double ld_stream(const double* p) { return __ldcs(p); }
__device__ __forceinline__ float ld_stream(const float* p) { return __ldcs(p); }
__device__ __forceinline__ int ld_stream(const int* p) { return __ldcs(p); }


// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
struct DeviceBuffer {
  void* ptr = nullptr;
  size_t bytes = 0;
};

struct axia_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;      // stream all work is issued on
  cudaStream_t own_stream = nullptr;  // the context's own stream
  int64_t launches = 0;               // kernels launched so far
  std::string last_error;
  int sm_count = 0;

  // mesh
  int nn = 0, reduced = 0, ngp = 0;
  int64_t n_nodes = 0, n_elem = 0;
  double nu = 0.0;
  double* d_coords = nullptr;   // [n_nodes*3]
  int32_t* d_conn = nullptr;    // [n_elem*nn]
  double* d_e = nullptr;        // [n_elem]

  // DOF map
  int64_t ndof = 0, n_free = 0;
  int32_t* d_ind_of = nullptr;  // [ndof], -1 prescribed
  double* d_u0 = nullptr;       // [ndof]
  bool any_u0 = false;

  // node incidence and adjacency
  int64_t* d_ne_ptr = nullptr;  // [n_nodes+1]
  int32_t* d_ne = nullptr;      // [n_elem*nn] packed element*32 + local node
  int64_t* d_adj_ptr = nullptr; // [n_nodes+1]
  int32_t* d_adj = nullptr;     // [n_adj]
  int32_t* d_adj_off = nullptr; // [n_adj] free-column offset of the block inside a row
  int32_t* d_node_rowlen = nullptr;  // [n_nodes]
  int64_t n_adj = 0;
  int max_adj = 0, max_inc = 0;

  // K_ff in CSR
  int64_t nnz = 0;
  int32_t* d_rowptr = nullptr;  // [n_free+1]
  int32_t* d_col = nullptr;     // [nnz]
  double* d_val = nullptr;      // [nnz]
  float* d_val32 = nullptr;     // [nnz] (mixed)
  double* d_diag = nullptr;     // [n_free]
  double* d_dinv = nullptr;     // [n_free]
  float* d_dinv32 = nullptr;    // [n_free]
  double* d_kfu0 = nullptr;     // [n_free]
  bool assembled = false, have32 = false, have_csr64 = false;

  // node-block (3x3) form of the full-DOF system: block rows padded to a
  // multiple of 4 blocks (pad column = the row's node, value 0) so that lanes
  // load 2 or 4 consecutive blocks of a row with one vector load per plane
  int32_t* d_adj_ptr32 = nullptr;  // [n_nodes+1] unpadded block-row starts
  int32_t* d_qptr = nullptr;       // [n_nodes+1] padded block-row starts (multiples of 4)
  int32_t* d_qadj = nullptr;       // [nbq] padded block columns
  int64_t nbq = 0;                 // padded block count
  double* d_bval64 = nullptr;      // [9][nbq]
  float* d_bval32 = nullptr;       // [9][nbq]
  double* d_bdinv64 = nullptr;     // [ndof]
  float* d_bdinv32 = nullptr;      // [ndof]
  bool have_bsr64 = false, have_bsr32 = false;
  float* d_bval32lo = nullptr;     // [9][nbq] fl32(K64 - K32) (AXIA_ASM_BSR32LO)
  bool have_bsr32lo = false;

  // symmetric node-block form of the FP32 matrix (AXIA_ASM_SYM32): every block
  // K_ab with b >= a stored once, in row a, as 10 floats (the 9 values row-major
  // and the block column as int bits); rows padded to an even block count (pad:
  // zero values, column = the row's node) so two blocks are five aligned float4.
  // The blocks with b < a are read through row a's lower list: (b, position of
  // K_ba in row b), K_ab = K_ba^T.
  int32_t* d_uptr = nullptr;       // [n_nodes+1] upper-block row starts (even)
  float* d_uval = nullptr;         // [nbu][10]
  int32_t* d_lptr = nullptr;       // [n_nodes+1] lower-list row starts
  int2* d_low = nullptr;           // [nbl] (b, position)
  int64_t nbu = 0, nbl = 0;
  bool have_sym32 = false;

  // element stiffness scratch
  double* d_ke = nullptr;
  size_t ke_elems = 0;
  bool ke_dw = false;           // d_ke holds double words (h, l) rather than FP64 (the last assembly)

  // solver vectors
  double* d_f = nullptr;        // [ndof]
  double* d_u = nullptr;        // [ndof]
  double* d_b = nullptr;        // [n_free]
  double* d_x = nullptr;
  double* d_r = nullptr;
  double* d_p = nullptr;
  double* d_q = nullptr;
  float* d_b32 = nullptr;
  float* d_x32 = nullptr;
  float* d_r32 = nullptr;
  float* d_p32 = nullptr;
  float* d_q32 = nullptr;
  double* d_partials = nullptr;
  double* d_totals = nullptr;
  size_t partial_slots = 0;
  GridBarrier* d_bar = nullptr;
  unsigned long long* d_first_bad = nullptr;  // first non-finite entry found by device_first_nonfinite
  DevStatus* d_status = nullptr;
  void* d_out = nullptr;        // PcgOut
  size_t vec_capacity = 0;
  // full-DOF vectors of the node-block solve
  double *d_bf = nullptr, *d_xf = nullptr, *d_rf = nullptr, *d_pf = nullptr, *d_qf = nullptr;
  float *d_xf32 = nullptr, *d_rf32 = nullptr, *d_pf32 = nullptr, *d_qf32 = nullptr, *d_zf32 = nullptr;
  size_t full_capacity = 0;
  // batched load cases ([ndof][32] blocks)
  double *d_mB = nullptr, *d_mX = nullptr;
  float *d_mX32 = nullptr, *d_mR32 = nullptr, *d_mP32 = nullptr, *d_mQ32 = nullptr;
  void* d_mout = nullptr;
  // segmented batched solve (double-word reliable updates): X as FP32 pairs and the kernel's state
  float *d_mXh = nullptr, *d_mXl = nullptr;
  size_t seg_capacity = 0;
  void* d_mstate = nullptr;
  size_t batch_capacity = 0;
  // block PCG of the load cases: W / Z block, Gram partials and results, small matrices
  float* d_mZ32 = nullptr;
  double* d_bpart = nullptr;    // [grid][3][32][32] per-block Gram partials
  double* d_bgram = nullptr;    // [4][32][32]: P^T Q, second Gram, W^T W, column norms
  float* d_bsmall = nullptr;    // [3][32][32]: alpha, beta, T (FP32 copies applied to the blocks)
  size_t bpart_capacity = 0;

  // multi-mesh solve: node ranges per mesh, CTA groups, captured graph
  std::vector<int64_t> mesh_node0;    // [n_meshes+1] first node of each mesh
  std::vector<int64_t> mesh_blocks;   // [n_meshes] node blocks of each mesh
  std::vector<int> multi_ctas;        // [n_meshes] blocks of each group
  unsigned char* d_mgroups = nullptr; // MeshGroup[n_meshes]
  int* d_mcta = nullptr;              // group of every block
  GridBarrier* d_mbars = nullptr;
  double* d_mtotals = nullptr;
  unsigned char* d_mouts = nullptr;   // PcgOut[n_meshes]
  int multi_grid = 0, multi_lanes = 0, multi_vec = 0;
  bool multi_coarse = false;          // groups planned for the two-level kernel
  int64_t graph_coarse = -1;    // coarse space the captured graph reads (its coarse_gen; -1: diagonal only)
  int64_t coarse_gen = 0;       // coarse spaces built so far (a new space gets new device arrays)
  int tuned_lanes = 0, tuned_vec = 0;  // node-block layout chosen by axia_gpu_autotune (0: none)
  int tuned_btc = 0, tuned_btu = 0;    // batched-kernel tile chosen by axia_gpu_autotune_batched (0: none)
  void* multi_graph = nullptr;        // cudaGraphExec_t
  const double* graph_f = nullptr;
  double* graph_u = nullptr;
  double graph_rtol = 0, graph_delta = 0;
  long long graph_max_iter = 0;

  // SIMP compliance state (forward -> backward)
  double* d_rho = nullptr;      // [n_elem]
  double* d_energy = nullptr;   // [n_elem]
  double* d_grad = nullptr;     // [n_elem]
  double simp_p = 3.0, simp_e0 = 1.0;
  bool have_forward = false;

  // stress recovery / reactions: per (element, local node) 6 stresses + 3 forces
  double* d_rec = nullptr;      // [n_elem*nn*9]

  // two-level preconditioner: coarse space of the mesh and its operator (coarse.cu)
  void* coarse = nullptr;       // CoarseState
  int64_t assemble_gen = 0;     // numeric assemblies so far (the operator follows K)

  double ms_setup = 0.0, ms_assemble = 0.0;
  double ms_element = 0.0, ms_gather = 0.0;  // kernel times of the last numeric assembly (CUDA events)
  // element stiffness arithmetic of C3D8 / C3D20 / C3D20R: double words on the
  // FP32 pipe (default) or the FP64 Gauss loop (axia_gpu_set_element_arith)
  bool element_fp64 = false;
  int64_t last_bad = -1;

  // device blocks of a released mesh state, kept for the next setup of the
  // same sizes (cudaFree of large blocks synchronises and costs milliseconds)
  std::unordered_map<void*, size_t> dev_bytes;  // live blocks from dev_alloc
  std::multimap<size_t, void*> dev_pool;         // released blocks by size
  size_t dev_pool_bytes = 0;
};

// set ctx->last_error and return code
int set_error(axia_ctx* ctx, int code, const std::string& msg);

#define AXIA_CUDA(ctx, call)                                                              \
  do {                                                                                    \
    cudaError_t _e = (call);                                                              \
    if (_e != cudaSuccess) {                                                              \
      return set_error((ctx), _e == cudaErrorMemoryAllocation ? AXIA_ERR_OOM : AXIA_ERR_CUDA, \
                       std::string(#call) + ": " + cudaGetErrorString(_e));              \
    }                                                                                     \
  } while (0)

#define AXIA_TRY(expr)      \
  do {                      \
    int _s = (expr);        \
    if (_s != AXIA_OK) return _s; \
  } while (0)

constexpr size_t DEV_POOL_CAP = (size_t)32 << 30;  // released bytes a context keeps at most

template <typename T>
int dev_alloc(axia_ctx* ctx, T** p, size_t count) {
  if (*p) {
    ctx->dev_bytes.erase((void*)*p);
    cudaFree(*p);
    *p = nullptr;
  }
  if (count == 0) count = 1;
  const size_t bytes = (count * sizeof(T) + 511) & ~(size_t)511;
  auto it = ctx->dev_pool.find(bytes);
  if (it != ctx->dev_pool.end()) {  // a released block of this size
    *p = (T*)it->second;
    ctx->dev_pool.erase(it);
    ctx->dev_pool_bytes -= bytes;
    ctx->dev_bytes[(void*)*p] = bytes;
    return AXIA_OK;
  }
  cudaError_t e = cudaMalloc((void**)p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    return set_error(ctx, AXIA_ERR_OOM, std::string("cudaMalloc ") + std::to_string(bytes) +
                                            " bytes: " + cudaGetErrorString(e));
  }
  ctx->dev_bytes[(void*)*p] = bytes;
  return AXIA_OK;
}

// Releases a block of the mesh state into the context's pool (the caller has
// synchronised the context's stream), or frees it when the pool is full.
template <typename T>
void dev_release(axia_ctx* ctx, T*& p) {
  if (!p) return;
  auto it = ctx->dev_bytes.find((void*)p);
  if (it != ctx->dev_bytes.end() && ctx->dev_pool_bytes + it->second <= DEV_POOL_CAP) {
    ctx->dev_pool.emplace(it->second, (void*)p);
    ctx->dev_pool_bytes += it->second;
  } else {
    cudaFree(p);
  }
  if (it != ctx->dev_bytes.end()) ctx->dev_bytes.erase(it);
  p = nullptr;
}

// frees every pooled block
inline void dev_pool_clear(axia_ctx* ctx) {
  for (auto& kv : ctx->dev_pool) cudaFree(kv.second);
  ctx->dev_pool.clear();
  ctx->dev_pool_bytes = 0;
}

template <typename T>
void dev_free(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

// exclusive scan of n int64 counts on the device (in place allowed), returns total
int device_exclusive_scan(axia_ctx* ctx, const int64_t* d_in, int64_t* d_out, int64_t n, int64_t* total);

// status word helpers
void coarse_release(axia_ctx* ctx);
int read_dev_status(axia_ctx* ctx, DevStatus* st_host);
int reset_dev_status(axia_ctx* ctx);
// Index of the first non-finite entry of the device vector d_v[0, n) (-1: all
// finite), checked on the device; one 8-byte read-back.
int device_first_nonfinite(axia_ctx* ctx, const double* d_v, int64_t n, int64_t* first);
