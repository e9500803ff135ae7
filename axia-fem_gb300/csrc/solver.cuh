// solver.cuh -- pieces shared by the CSR (pcg.cu) and node-block (bsr.cu)
// persistent Krylov kernels: block partial sums, the PCG result record and
// the CSR argument pack.
#pragma once

#include "common.cuh"

constexpr int PCG_THREADS = 512;
int pcg_lanes_for(const axia_ctx* ctx, bool fp32, int requested);
constexpr int S_PQ = 0, S_RR = 1, S_RZ = 2, N_SLOTS = 3;

// result of one persistent solve, written by block 0
struct PcgOut {
  long long iters;
  double residual;
  double bnorm;
  int status;
  int updates;
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
  double* totals;    // [N_SLOTS]
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
// (block `rank` of a group of nblk blocks; the whole grid by default)
template <typename A>
__device__ __forceinline__ void block_partials(A v0, A v1, int nv, double* partials, int slot0, int slot1,
                                               unsigned nblk = 0, unsigned rank = 0) {
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
      if (nblk == 0) {
        nblk = gridDim.x;
        rank = blockIdx.x;
      }
      partials[slot0 * nblk + rank] = (double)a0;
      if (nv > 1) partials[slot1 * nblk + rank] = (double)a1;
    }
  }
}

__device__ __forceinline__ double total(const double* totals, int slot) { return __ldcg(totals + slot); }


// ---------------------------------------------------------------------------
// Node-block (3x3) matrix and the mixed-precision argument pack (bsr.cu)
// ---------------------------------------------------------------------------
template <typename V>
struct BsrMat {
  int n_nodes;
  const int* adj_ptr;  // [n_nodes+1]
  const int* adj;      // [nb]
  const V* val;        // [9][nb]
  long long nb;
};

// Symmetric FP32 node-block form (axia_ctx::d_uval ...): upper blocks of row a
// at [uptr[a], uptr[a+1]) as 10 floats each (9 values, column bits), lower
// neighbours of row a at [lptr[a], lptr[a+1]) as (b, position of K_ba).
struct SymMat {
  int n_nodes;
  const int* uptr;
  const float* uval;
  const int* lptr;
  const int2* low;
};

// one system of a multi-mesh solve: its block rows and its blocks
struct MeshGroup {
  int node0, node1;   // block rows [node0, node1)
  int cta0, ncta;     // blocks [cta0, cta0 + ncta) of the launch
  long long part_off; // offset of its partial-sum area
  int chunk0, chunk1; // its restriction chunks (two-level preconditioner)
  int row0, row1;     // its coarse unknowns
  int col0, ldm;      // its block of the coarse inverse: first unknown, padded size
  long long moff;     // element offset of that block
};
constexpr int GROUP_SLOTS = 4;  // partial-sum slots per group: S_PQ, S_RR, S_RZ, S_RC

constexpr int COARSE_MAX = 4096;    // coarse unknowns (6 per subdomain, padded to 64)
constexpr int COARSE_CHUNK = 256;   // nodes per restriction chunk
constexpr int S_RC = 3;             // partial-sum slot of r_c . y

struct CoarseArgs {
  int n_sub;             // subdomains (0: no coarse space)
  int nc;                // 6 n_sub
  int row0, row1;        // the coarse unknowns whose rows of y = M r_c this launch (group) computes
  int chunk_lo, chunk_hi;  // the restriction chunks this launch (group) handles
  int ncp;               // length of rc / yc (one block: nc rounded up to a multiple of 64)
  int col0, ldm;         // the block of M this launch (group) reads: unknowns col0 .., row stride ldm
  int n_chunks;
  const int* sub_node;   // [n_nodes] nodes by subdomain, ascending within each
  const int4* chunk;     // [n_chunks] (subdomain, first, end) ranges of sub_node
  const int* chunk_ptr;  // [n_sub + 1] chunks of each subdomain
  const float4* geo;     // [n_nodes] (x_a - c_I) / h, .w = bits (I << 3 | free-DOF mask)
  const float* minv;     // this launch's block of M: [rows][ldm], row r at (r - col0) ldm, zero in the padding
  float* part;           // [n_chunks][6] restriction partials
  float* rc;             // [ncp] restricted residual Z^T r (zero in the padding)
  int* cnt;              // [n_sub] chunks of each subdomain done (reset by the last)
  float* yc;             // [ncp] coarse correction y = M r_c
  // 32 load cases at once (batch.cu): [n_chunks][6][32], [ncp][32], [ncp][32]
  float* part_m;
  float* rc_m;
  float* yc_m;
};

struct BsrReliableArgs {
  BsrMat<float> M32;
  SymMat S32;        // the FP32 matrix in symmetric storage (kernels instantiated with SYM)
  BsrMat<double> M64;
  int nd;
  const float* dinv32;
  const double* b;
  double* x;
  float* x32;
  float* r32;
  float* p32;
  float* q32;
  float* z32;
  double* partials;
  double* totals;
  GridBarrier* bar;
  DevStatus* st;
  PcgOut* out;
  double tol;
  double delta;
  long long max_iter;
  unsigned long long limit_ns;
  CoarseArgs C;      // two-level preconditioner (n_sub = 0: Jacobi only)
};

BsrReliableArgs make_reliable_args(axia_ctx* ctx, double rtol, double delta, long long max_iter);
int group_kernel_capacity(axia_ctx* ctx, int lanes, int vec, int* per_sm, bool coarse = false);
void group_layout(const axia_ctx* ctx, int lanes_req, int vec_req, int* lanes, int* vec);
int launch_group_reliable(axia_ctx* ctx, BsrReliableArgs& P, const MeshGroup* groups, const int* cta_group,
                          GridBarrier* bars, double* totals4, PcgOut* outs, int grid, int lanes, int vec, bool coarse = false);
int launch_full_rhs(axia_ctx* ctx, const double* d_f);
int launch_full_reconstruct(axia_ctx* ctx, double* d_u);
int prepare_full_buffers(axia_ctx* ctx);

// Sorted (key, value) pairs and their runs of equal keys (triplets.cu).
struct Runs {
  uint64_t* key = nullptr;  // sorted keys
  double* val = nullptr;    // values in sorted order
  int64_t* head = nullptr;  // first position of each run
  int64_t nv = 0, n_runs = 0;
  void release() {
    dev_free(key);
    dev_free(val);
    dev_free(head);
    n_runs = nv = 0;
  }
};
int sort_runs(axia_ctx* ctx, const uint64_t* dk, const double* dv, int64_t nt, int64_t nv, int end_bit, Runs* out);
int key_bits(uint64_t max_key);
int csr_from_runs(axia_ctx* ctx, int64_t n, const Runs& R, bool fp32);
int vector_from_runs(axia_ctx* ctx, int64_t n, const Runs& R, double* d_out);

// Device copy of a DOF map (T, u0) and the reduced right-hand side (reduce.cu).
struct ReducedSystem {
  int64_t n_full = 0, n_ind = 0;
  int64_t* t_ptr = nullptr;
  int64_t* t_col = nullptr;
  double* t_val = nullptr;
  double* u0 = nullptr;
  double* rhs = nullptr;
  void release() {
    dev_free(t_ptr);
    dev_free(t_col);
    dev_free(t_val);
    dev_free(u0);
    dev_free(rhs);
  }
};
int reduce_system(axia_ctx* ctx, const axia_dofmap* map, int64_t nt, const int64_t* h_i, const int64_t* h_j,
                  const double* h_v, const double* h_f, bool fp32, ReducedSystem* S);
int reconstruct_system(axia_ctx* ctx, const ReducedSystem& S, const double* d_x, double* d_u);

// ---------------------------------------------------------------------------
// Host helpers for the persistent launches
// ---------------------------------------------------------------------------
inline int coop_grid(axia_ctx* ctx, const void* kern, int n, int* grid_out, size_t dyn_smem = 0) {
  int per_sm = 0;
  AXIA_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, PCG_THREADS, dyn_smem));
  if (per_sm < 1) return set_error(ctx, AXIA_ERR_CUDA, "PCG kernel does not fit on an SM");
  int grid = per_sm * ctx->sm_count;
  int need = (n + PCG_THREADS - 1) / PCG_THREADS;
  grid = std::max(1, std::min(grid, std::max(need, ctx->sm_count)));
  if ((size_t)grid * N_SLOTS > ctx->partial_slots) return set_error(ctx, AXIA_ERR_STATE, "partials buffer too small");
  *grid_out = grid;
  return AXIA_OK;
}


// one persistent launch bracketed by CUDA events on the launching stream
template <typename F>
inline int timed_launch(axia_ctx* ctx, axia_solve_info* info, F&& launch) {
  cudaEvent_t a, b;
  AXIA_CUDA(ctx, cudaEventCreate(&a));
  AXIA_CUDA(ctx, cudaEventCreate(&b));
  cudaEventRecord(a, ctx->stream);
  int st = launch();
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


inline int read_out(axia_ctx* ctx, PcgOut* o) {
  AXIA_CUDA(ctx, cudaMemcpyAsync(o, ctx->d_out, sizeof(PcgOut), cudaMemcpyDeviceToHost, ctx->stream));
  AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  DevStatus hs;
  AXIA_TRY(read_dev_status(ctx, &hs));
  if (hs.timeout) return set_error(ctx, AXIA_ERR_TIMEOUT, "a grid barrier of the PCG kernel ran past its time limit");
  return AXIA_OK;
}


inline int status_error(axia_ctx* ctx, const PcgOut& o) {
  if (o.status == AXIA_ERR_NOT_CONVERGED)
    return set_error(ctx, o.status, "CG did not converge (residual " + std::to_string(o.residual) + " after " +
                                        std::to_string(o.iters) + " iterations)");
  if (o.status == AXIA_ERR_ZERO_PIVOT) return set_error(ctx, o.status, "CG: zero pivot, matrix not positive definite");
  return set_error(ctx, o.status, "CG: non-finite iterate");
}


