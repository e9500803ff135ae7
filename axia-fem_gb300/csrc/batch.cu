// batch.cu -- many load cases on one mesh in one persistent launch.
//
// 32 right-hand sides share every sweep over the node-block matrix: the
// vectors are stored [nd][32] (the 32 load cases of a DOF contiguous), a warp
// owns one block row, its four 8-lane groups walk the row's blocks, and each
// lane applies the 3x3 block to 4 load cases with 16-byte vector loads, so a
// block's 9 values are read once for 32 products.  Every column runs its own
// Jacobi-PCG recurrence (solver/src/linalg.rs:199-259: its own alpha, beta,
// convergence test) on the FP32 node-block matrix, with FP64 reliable updates
// (x += x32, r = b - K x in FP64 for all columns) when every active column's
// FP32 residual has dropped by delta, or one has reached the tolerance.
// A converged column is frozen (alpha = beta = 0).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>

#include "coarse.cuh"
#include "dword.cuh"

namespace {

constexpr int NR = 32;   // load cases per column block
constexpr int CPL = 4;   // load cases per lane
constexpr int LPG = 8;   // lanes per group (LPG * CPL = NR)

template <typename V>
struct BsrMatM {
  int n_nodes;
  const int* adj_ptr;
  const int* adj;
  const V* val;  // [9][nb]
  long long nb;
};

__device__ __forceinline__ void ld4(const float* p, float v[4]) {
  const float4 t = *reinterpret_cast<const float4*>(p);
  v[0] = t.x, v[1] = t.y, v[2] = t.z, v[3] = t.w;
}
__device__ __forceinline__ void ld4(const double* p, double v[4]) {
  const double2 a = *reinterpret_cast<const double2*>(p), b = *reinterpret_cast<const double2*>(p + 2);
  v[0] = a.x, v[1] = a.y, v[2] = b.x, v[3] = b.y;
}
__device__ __forceinline__ void st4(float* p, const float v[4]) {
  *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void st4(double* p, const double v[4]) {
  *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
  *reinterpret_cast<double2*>(p + 2) = make_double2(v[2], v[3]);
}

// Rows of at most STAGE_B blocks (C3D8 rows have up to 27) are staged: while a
// warp computes one block row, the matrix values and block columns of its
// next row are copied to shared memory asynchronously (cp.async, 4 bytes per
// lane and array), so a step of the row loop waits only for the vector rows
// (mostly L1 / L2 hits), not for the matrix stream from DRAM.  Longer rows
// read their values from the matrix planes.
constexpr int STAGE_B = 28;
struct RowStage {
  float v[9][STAGE_B];
  int adj[STAGE_B];
};
constexpr size_t STAGE_BYTES = sizeof(RowStage) * 2 * (PCG_THREADS / 32);  // two per warp

__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Starts the copy of row a into st (nothing for a >= n_nodes or a long row)
// and closes the lane's copy group.
__device__ __forceinline__ void stage_row(int a, int lane, const BsrMatM<float>& M, RowStage* st) {
  if (a < M.n_nodes) {
    const int beg = __ldg(M.adj_ptr + a), len = __ldg(M.adj_ptr + a + 1) - beg;
    if (len <= STAGE_B && lane < len) {
#pragma unroll
      for (int k = 0; k < 9; ++k) cp_async4(&st->v[k][lane], M.val + (long long)k * M.nb + beg + lane);
      cp_async4(&st->adj[lane], M.adj + beg + lane);
    }
  }
  cp_async_commit();
}

// ---------------------------------------------------------------------------
// Tiled row product for the FP32 SpMV, the shape picked by the batch
// autotuner: TC load cases per lane (1, 2 or 4: a group of 32 / TC lanes
// covers the 32 cases, a warp holds TC groups that take interleaved blocks of
// the row) and TU blocks per group and step, whose vector rows (3 x TC floats
// per lane and block) are all requested before any is used, so a lane keeps
// 3 TU loads in flight instead of waiting for one block at a time.  The
// result for cases TC cl .. TC cl + TC - 1 is valid in the lanes of group 0
// (lane < 32 / TC) after the call.
// ---------------------------------------------------------------------------
template <int TC>
__device__ __forceinline__ void ldc(const float* p, float (&v)[TC]) {
  if constexpr (TC == 4) {
    const float4 t = *reinterpret_cast<const float4*>(p);
    v[0] = t.x, v[1] = t.y, v[2] = t.z, v[3] = t.w;
  } else if constexpr (TC == 2) {
    const float2 t = *reinterpret_cast<const float2*>(p);
    v[0] = t.x, v[1] = t.y;
  } else {
    v[0] = *p;
  }
}

template <int TC>
__device__ __forceinline__ void stc(float* p, const float (&v)[TC]) {
  if constexpr (TC == 4)
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  else if constexpr (TC == 2)
    *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
  else
    *p = v[0];
}

// values of block s: from the row's staging (staged) or the matrix planes
template <int TC, int TU, bool STAGED>
__device__ __forceinline__ void row_tile(int a, int len, int lane, const RowStage* st, const BsrMatM<float>& M,
                                         const float* X, float (&y)[3][TC]) {
  constexpr int LG = NR / TC, G = 32 / LG;
  const int cl = lane % LG, grp = lane / LG;
  const int beg = STAGED ? 0 : __ldg(M.adj_ptr + a);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int c = 0; c < TC; ++c) y[i][c] = 0.f;
  for (int s0 = grp; s0 < len; s0 += G * TU) {
    float x[TU][3][TC];
#pragma unroll
    for (int u = 0; u < TU; ++u) {
      const int s = s0 + u * G;
      if (s < len) {
        const int b = STAGED ? st->adj[s] : ld_stream(M.adj + beg + s);
#pragma unroll
        for (int j = 0; j < 3; ++j) ldc<TC>(X + (size_t)(3 * b + j) * NR + TC * cl, x[u][j]);
      } else {
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
          for (int c = 0; c < TC; ++c) x[u][j][c] = 0.f;
      }
    }
#pragma unroll
    for (int u = 0; u < TU; ++u) {
      const int s = s0 + u * G;
      if (s < len) {
        float v[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) v[k] = STAGED ? st->v[k][s] : ld_stream(M.val + (long long)k * M.nb + beg + s);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int c = 0; c < TC; ++c)
            y[i][c] = fmaf(v[3 * i], x[u][0][c], fmaf(v[3 * i + 1], x[u][1][c], fmaf(v[3 * i + 2], x[u][2][c], y[i][c])));
      }
    }
  }
#pragma unroll
  for (int o = LG; o < 32; o <<= 1)
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int c = 0; c < TC; ++c) y[i][c] += __shfl_xor_sync(0xffffffffu, y[i][c], o);
}

// Y[3a+i][4 cl + 2 h + c], c = 0, 1: two of the lane's four load cases in FP64.
// The FP64 residual of a reliable update runs in two such halves so that the
// kernel fits the register budget of two blocks per SM.
__device__ __forceinline__ void bsr_row_multi_half(int a, int lane, const BsrMatM<double>& M, const double* X, int h,
                                                   double y[3][2]) {
  const int cl = lane % LPG, grp = lane / LPG;
#pragma unroll
  for (int i = 0; i < 3; ++i) y[i][0] = y[i][1] = 0.0;
  const int beg = __ldg(M.adj_ptr + a), end = __ldg(M.adj_ptr + a + 1);
  int b = beg + grp < end ? ld_stream(M.adj + beg + grp) : 0;
  for (int s = beg + grp; s < end; s += 32 / LPG) {
    const int b_next = s + 32 / LPG < end ? ld_stream(M.adj + s + 32 / LPG) : 0;
    double v[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) v[k] = ld_stream(M.val + (long long)k * M.nb + s);
    double x[3][2];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double2 t = *reinterpret_cast<const double2*>(X + (size_t)(3 * b + j) * NR + CPL * cl + 2 * h);
      x[j][0] = t.x;
      x[j][1] = t.y;
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int c = 0; c < 2; ++c)
        y[i][c] = fma(v[3 * i], x[0][c], fma(v[3 * i + 1], x[1][c], fma(v[3 * i + 2], x[2][c], y[i][c])));
    b = b_next;
  }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      y[i][c] += __shfl_xor_sync(0xffffffffu, y[i][c], 8);
      y[i][c] += __shfl_xor_sync(0xffffffffu, y[i][c], 16);
    }
}

// Per-column partial sums of this block: v[c] is this thread's contribution
// to column TC*(tid % (32/TC))+c (TC = 4: the float4 layout of the vector
// phases).  Written to partials[(slot0 + col) * G + block].
// one scratch for every instantiation of block_partials_cols (a __shared__
// array inside the template is allocated once per instantiation: 8 KB each)
__device__ __forceinline__ double (*cols_scratch())[NR] {
  __shared__ double s_cols[PCG_THREADS / 32][NR];
  return s_cols;
}

template <typename A, int TC = CPL>
__device__ __forceinline__ void block_partials_cols(const A (&v)[TC], double* partials, int slot0) {
  constexpr int LG = NR / TC;
  double (*s_cols)[NR] = cols_scratch();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  double t[TC];
#pragma unroll
  for (int c = 0; c < TC; ++c) {
    t[c] = (double)v[c];
#pragma unroll
    for (int o = LG; o < 32; o <<= 1) t[c] += __shfl_xor_sync(0xffffffffu, t[c], o);
  }
  if (lane < LG) {
#pragma unroll
    for (int c = 0; c < TC; ++c) s_cols[warp][TC * lane + c] = t[c];
  }
  __syncthreads();
  if (threadIdx.x < NR) {
    double s = 0.0;
    for (int w = 0; w < nw; ++w) s += s_cols[w][threadIdx.x];
    partials[(size_t)(slot0 + threadIdx.x) * gridDim.x + blockIdx.x] = s;
  }
}

// Reduce-and-sync over nv partial slots; the last block to arrive sums them
// (one warp per slot, ascending block order) and publishes totals[slot0..].
__device__ __forceinline__ bool grid_reduce_sync_wide(GridBarrier* bar, DevStatus* st, unsigned long long limit_ns,
                                                      const double* partials, double* totals, int slot0, int nv) {
  __shared__ int s_last, s_ok;
  __shared__ unsigned s_gen;
  __syncthreads();
  if (threadIdx.x == 0) {
    int last;
    s_gen = barrier_arrive(bar, gridDim.x, &last);
    s_last = last;
  }
  __syncthreads();
  int ok = 1;
  if (s_last) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int k = warp; k < nv; k += nw) {
      const int cnt = lane < (int)gridDim.x ? ((int)gridDim.x - lane + 31) / 32 : 0;
      double a = ldcg_sum(partials + (size_t)(slot0 + k) * gridDim.x + lane, 32, cnt);
      a = warp_sum(a);
      if (lane == 0) totals[slot0 + k] = a;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      barrier_release(bar, s_gen);
    }
  } else if (threadIdx.x == 0) {
    ok = barrier_wait(bar, st, limit_ns, s_gen);
  }
  if (threadIdx.x == 0) s_ok = ok;
  __syncthreads();
  return s_ok != 0;
}

struct MultiOut {
  long long iters;
  int updates;
  int status;
  double bnorm[NR];
  double residual[NR];
  long long col_iters[NR];
};

// The per-case state of pcg_bsr_multi_kernel between launches when it runs
// in segments (MultiArgs::split): the kernel stops at each reliable update,
// the update runs as its own launches, and the kernel resumes from here.
struct BatchState {
  long long it, iters;
  int updates;
  int phase;  // 1: stopped for a reliable update, 0: finished
  double rz[NR], bnorm[NR], rmax[NR], res[NR], rrec[NR];
  int active[NR];
  long long citers[NR];
};

struct MultiArgs {
  BsrMatM<float> M32;
  BsrMatM<double> M64;
  int nd;
  const float* dinv32;  // [nd]
  const double* B;      // [nd][NR]
  double* X;            // [nd][NR]
  float* X32;
  float* R32;
  float* P32;
  float* Q32;
  double* partials;     // [>= 2 NR][G]
  double* totals;       // [>= 2 NR]
  GridBarrier* bar;
  DevStatus* st;
  MultiOut* out;
  double tol;
  double delta;
  long long max_iter;
  unsigned long long limit_ns;
  CoarseArgs C;         // two-level preconditioner (n_sub = 0: Jacobi only)
  BatchState* state = nullptr;
  int split = 0;        // stop at every reliable update (state saved, phase 1)
  int resume = 0;       // start from state, after an update whose |r|^2 and r.D^-1 r are in totals
};

constexpr int SL_A = 0, SL_B = NR;  // two banks of NR slots

// ---------------------------------------------------------------------------
// Two-level preconditioner for 32 columns (the single-column form is in
// coarse.cuh): restriction per chunk of a subdomain's nodes with four 8-lane
// groups taking four nodes at a time (lane cl of a group: columns 4cl..4cl+3),
// the last warp of a subdomain summing its chunk partials in chunk order;
// y = M r_c as tasks (row, column quad) with lanes over the coarse unknowns;
// the prolongation inside the search-direction update.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void coarse_restrict_m(const CoarseArgs& C, const float* R, int gwarp, int nwarps,
                                                  int lane) {
  const int cl = lane % LPG, grp = lane / LPG;
  for (int ci = C.chunk_lo + gwarp; ci < C.chunk_hi; ci += nwarps) {
    const int4 ch = C.chunk[ci];
    float v[6][CPL];
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
      for (int c = 0; c < CPL; ++c) v[i][c] = 0.f;
#pragma unroll 2
    for (int k = ch.y + grp; k < ch.z; k += 32 / LPG) {
      const int a = __ldg(C.sub_node + k);
      const float4 g = __ldg(C.geo + a);
      const unsigned m = geo_bits(g);
      float r[3][CPL];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        if ((m >> d) & 1u) {
          ld4(R + (size_t)(3 * a + d) * NR + CPL * cl, r[d]);
        } else {
#pragma unroll
          for (int c = 0; c < CPL; ++c) r[d][c] = 0.f;
        }
      }
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        v[0][c] += r[0][c];
        v[1][c] += r[1][c];
        v[2][c] += r[2][c];
        v[3][c] = fmaf(g.y, r[2][c], fmaf(-g.z, r[1][c], v[3][c]));
        v[4][c] = fmaf(g.z, r[0][c], fmaf(-g.x, r[2][c], v[4][c]));
        v[5][c] = fmaf(g.x, r[1][c], fmaf(-g.y, r[0][c], v[5][c]));
      }
    }
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        v[i][c] += __shfl_xor_sync(0xffffffffu, v[i][c], 8);
        v[i][c] += __shfl_xor_sync(0xffffffffu, v[i][c], 16);
      }
    if (grp == 0)
#pragma unroll
      for (int i = 0; i < 6; ++i) st4(C.part_m + ((size_t)ci * 6 + i) * NR + CPL * cl, v[i]);
    __threadfence();
    __syncwarp();
    const int I = ch.x, c0 = __ldg(C.chunk_ptr + I), c1 = __ldg(C.chunk_ptr + I + 1);
    int last = 0;
    if (lane == 0) last = atomicAdd(C.cnt + I, 1) == c1 - c0 - 1;
    last = __shfl_sync(0xffffffffu, last, 0);
    if (last) {
      __threadfence();
#pragma unroll
      for (int i = 0; i < 6; ++i)
        C.rc_m[(size_t)(6 * I + i) * NR + lane] =
            ldcg_sum(C.part_m + ((size_t)c0 * 6 + i) * NR + lane, (size_t)6 * NR, c1 - c0);
      if (lane == 0) atomicExch(C.cnt + I, 0);
    }
  }
}

// Y = M R_c; per column r_c . y into partials[(slot0 + col) * G + block].
// Tasks of 16 rows go to the blocks in turn; a thread owns one (row, load
// case).  The task walks the columns of M in tiles of 64: the tile of R_c
// (64 x 32, contiguous) and the 16 x 64 tile of M are copied into a 3-stage
// shared-memory ring with cp.async, two tiles ahead of the one being summed,
// so a task keeps ~24 KB in flight instead of waiting one memory round trip
// per tile.  `ring` is COARSE_RING_FLOATS of 16-byte aligned shared memory.
// The per-column sums run over the block's tasks and rows in a fixed order.
constexpr int CS_TJ = 64;                          // columns of M per tile
constexpr int CS_TR = PCG_THREADS / NR;            // rows per task (16)
constexpr int CS_STAGE = CS_TJ * NR + CS_TR * CS_TJ;  // floats per stage: R_c tile + M tile
constexpr int COARSE_RING_FLOATS = 3 * CS_STAGE;

// dynamic shared memory of the 32-case kernel: the row staging of the SpMV
// phase and the coarse solve's ring take turns in it
constexpr size_t DYN_BYTES =
    STAGE_BYTES > COARSE_RING_FLOATS * sizeof(float) ? STAGE_BYTES : COARSE_RING_FLOATS * sizeof(float);

__device__ __forceinline__ void cp_async16(float* smem, const float* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}

__device__ __forceinline__ void coarse_solve_m(const CoarseArgs& C, float* ring, double* partials, int slot0) {
  __shared__ float s_prod[PCG_THREADS];
  __shared__ float s_cc[NR];
  const int r = threadIdx.x / NR, c = threadIdx.x % NR;
  if (threadIdx.x < NR) s_cc[threadIdx.x] = 0.f;
  const int ntask = (C.nc + CS_TR - 1) / CS_TR;
  const int nt = C.ldm / CS_TJ;  // tiles per row of M (ldm is a multiple of 64; zero past nc)
  for (int task = blockIdx.x; task < ntask; task += gridDim.x) {
    const int i0 = task * CS_TR;
    // thread t copies 16 bytes of the R_c tile and (t < 256) 16 bytes of the M tile
    auto issue = [&](int t) {
      if (t < nt) {
        float* st = ring + (t % 3) * CS_STAGE;
        const int jj = threadIdx.x >> 3, cc = 4 * (threadIdx.x & 7);
        cp_async16(st + jj * NR + cc, C.rc_m + (size_t)(t * CS_TJ + jj) * NR + cc);
        if (threadIdx.x < CS_TR * CS_TJ / 4) {
          const int rr = threadIdx.x >> 4, kk = 4 * (threadIdx.x & 15);
          cp_async16(st + CS_TJ * NR + rr * CS_TJ + kk, C.minv + (size_t)(i0 + rr) * C.ldm + t * CS_TJ + kk);
        }
      }
      asm volatile("cp.async.commit_group;" ::: "memory");
    };
    __syncthreads();  // the ring is free (the previous task's readers are done)
    issue(0);
    issue(1);
    float y = 0.f;
    for (int t = 0; t < nt; ++t) {
      asm volatile("cp.async.wait_group 1;" ::: "memory");  // tile t has landed
      __syncthreads();
      issue(t + 2);  // into the stage tile t - 1 used; every thread is past it
      const float* st = ring + (t % 3) * CS_STAGE;
      const float* mt = st + CS_TJ * NR + r * CS_TJ;
#pragma unroll 8
      for (int jj = 0; jj < CS_TJ; ++jj) y = fmaf(mt[jj], st[jj * NR + c], y);
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    const int i = i0 + r;
    float prod = 0.f;
    if (i < C.nc) {
      C.yc_m[(size_t)i * NR + c] = y;
      prod = __ldcg(C.rc_m + (size_t)i * NR + c) * y;
    }
    s_prod[threadIdx.x] = prod;
    __syncthreads();
    if (threadIdx.x < NR) {
      float sum = s_cc[threadIdx.x];
      for (int q = 0; q < CS_TR; ++q) sum += s_prod[q * NR + threadIdx.x];
      s_cc[threadIdx.x] = sum;
    }
  }
  __syncthreads();
  if (threadIdx.x < NR) partials[(size_t)(slot0 + threadIdx.x) * gridDim.x + blockIdx.x] = (double)s_cc[threadIdx.x];
}

// coarse part of z at DOF row `row`, columns c0..c0+3
__device__ __forceinline__ void coarse_prolong_m(const CoarseArgs& C, long long row, int c0, float zc[CPL]) {
  const int a = (int)(row / 3), d = (int)(row - 3LL * a);
  const float4 g = __ldg(C.geo + a);
  const unsigned m = geo_bits(g);
#pragma unroll
  for (int c = 0; c < CPL; ++c) zc[c] = 0.f;
  if (!((m >> d) & 1u)) return;
  const float* Y = C.yc_m + (size_t)(6 * (m >> 3)) * NR + c0;
  float t[CPL], u[CPL], w[CPL];
  float cu, cw;
  if (d == 0) {
    ld4(Y, t), ld4(Y + 4 * NR, u), ld4(Y + 5 * NR, w), cu = g.z, cw = -g.y;
  } else if (d == 1) {
    ld4(Y + NR, t), ld4(Y + 3 * NR, u), ld4(Y + 5 * NR, w), cu = -g.z, cw = g.x;
  } else {
    ld4(Y + 2 * NR, t), ld4(Y + 3 * NR, u), ld4(Y + 4 * NR, w), cu = g.y, cw = -g.x;
  }
#pragma unroll
  for (int c = 0; c < CPL; ++c) zc[c] = fmaf(cu, u[c], fmaf(cw, w[c], t[c]));
}

// the coarse half of the preconditioner for the current R32: restriction,
// barrier, Y = M R_c and the per-column r . Z y reduced into totals[SL_A..]
__device__ __forceinline__ bool coarse_step_m(const MultiArgs& P, int gwarp, int nwarps, int lane, float* ring) {
  coarse_restrict_m(P.C, P.R32, gwarp, nwarps, lane);
  if (!grid_sync(P.bar, P.st, P.limit_ns)) return false;
  coarse_solve_m(P.C, ring, P.partials, SL_A);
  return grid_reduce_sync_wide(P.bar, P.st, P.limit_ns, P.partials, P.totals, SL_A, NR);
}

template <bool COARSE, int TC, int TU>
__global__ void __launch_bounds__(PCG_THREADS, 2) pcg_bsr_multi_kernel(MultiArgs P) {
  extern __shared__ __align__(16) RowStage s_stage[];  // DYN_BYTES: row staging, or the coarse solve's ring
  float* const ring = reinterpret_cast<float*>(s_stage);
  __shared__ double s_rz[NR], s_bnorm[NR], s_rmax[NR], s_res[NR];
  __shared__ float s_alpha[NR], s_beta[NR];
  __shared__ int s_active[NR], s_flag, s_restart[NR];
  __shared__ double s_rrec[NR];  // recurrence |r| of each case when the last update was triggered
  __shared__ long long s_citers[NR];
  const int nd = P.nd, n_nodes = P.M32.n_nodes;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31;
  const int gwarp = tid >> 5, nwarps = nth >> 5;
  const int cq = tid % LPG;            // this thread's column quad in the vector phases
  const long long nq = (long long)nd * LPG;  // float4 chunks of an [nd][NR] vector
  // the bookkeeping after a reliable update whose |r|^2 (slots SL_A) is in
  // totals.  A case whose true residual came back more than twice its
  // recurrence residual restarts its search direction (beta = 0): the
  // replaced residual no longer fits the old directions, and carrying them on
  // let the FP32 recurrence of an ill-conditioned case wander instead of
  // converging.
  auto after_update = [&](int& updates) {
    ++updates;
    if (threadIdx.x < NR) {
      const int c = threadIdx.x;
      const double rn = sqrt(__ldcg(P.totals + SL_A + c));
      s_restart[c] = 0;
      if (s_active[c]) {
        s_restart[c] = rn > 2.0 * s_rrec[c];
        s_res[c] = rn;
        s_rmax[c] = rn;
        if (rn <= P.tol * s_bnorm[c]) s_active[c] = 0;  // converged
      }
    }
    __syncthreads();
  };
  // the end of an iteration: the coarse correction of r, beta, p = z + beta p
  auto iteration_tail = [&]() -> bool {
    if constexpr (COARSE) {
      if (!coarse_step_m(P, gwarp, nwarps, lane, ring)) return false;
    }
    if (threadIdx.x < NR) {
      const int c = threadIdx.x;
      double rzn = __ldcg(P.totals + SL_B + c);
      if constexpr (COARSE) rzn += __ldcg(P.totals + SL_A + c);
      s_beta[c] = s_active[c] && !s_restart[c] ? (float)(rzn / s_rz[c]) : 0.f;
      s_restart[c] = 0;
      s_rz[c] = rzn;
    }
    __syncthreads();
    for (long long q = tid; q < nq; q += nth) {
      const long long row = q / LPG;
      const int c0 = CPL * (int)(q % LPG);
      float p[CPL], r[CPL], zc[CPL] = {0.f, 0.f, 0.f, 0.f};
      ld4(P.P32 + q * CPL, p);
      ld4(P.R32 + q * CPL, r);
      if constexpr (COARSE) coarse_prolong_m(P.C, row, c0, zc);
      const float di = P.dinv32[row];
#pragma unroll
      for (int c = 0; c < CPL; ++c)
        p[c] = s_active[c0 + c] ? fmaf(s_beta[c0 + c], p[c], fmaf(r[c], di, zc[c])) : 0.f;
      st4(P.P32 + q * CPL, p);
    }
    return grid_sync(P.bar, P.st, P.limit_ns);
  };
  long long it0 = 0, iters0 = 0;
  int updates0 = 0;
  if (P.resume) {  // the rest of the iteration that stopped for the update
    if (threadIdx.x < NR) {
      const int c = threadIdx.x;
      s_rz[c] = P.state->rz[c];
      s_bnorm[c] = P.state->bnorm[c];
      s_rmax[c] = P.state->rmax[c];
      s_res[c] = P.state->res[c];
      s_active[c] = P.state->active[c];
      s_citers[c] = P.state->citers[c];
      s_rrec[c] = P.state->rrec[c];
      s_restart[c] = 0;
    }
    it0 = P.state->it + 1;
    iters0 = P.state->iters;
    updates0 = P.state->updates;
    __syncthreads();
    after_update(updates0);
    if (!iteration_tail()) return;
  }
  // init: x = 0, r32 = b, p = z = r32 / diag, per-column r.z and b.b
  if (!P.resume) {
    float rz_p[CPL] = {0, 0, 0, 0};
    double bb_p[CPL] = {0, 0, 0, 0};
    for (long long q = tid; q < nq; q += nth) {
      const long long row = q / LPG;
      double bv[CPL];
      ld4(P.B + q * CPL, bv);
      const float di = P.dinv32[row];
      float r[CPL], z[CPL];
      const double zero4[CPL] = {0, 0, 0, 0};
      const float fz4[CPL] = {0, 0, 0, 0};
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        r[c] = (float)bv[c];
        z[c] = r[c] * di;
        rz_p[c] = fmaf(r[c], z[c], rz_p[c]);
        bb_p[c] = fma(bv[c], bv[c], bb_p[c]);
      }
      st4(P.X + q * CPL, zero4);
      st4(P.X32 + q * CPL, fz4);
      st4(P.R32 + q * CPL, r);
      st4(P.P32 + q * CPL, z);
    }
    block_partials_cols<double>(bb_p, P.partials, SL_A);
    __syncthreads();
    block_partials_cols<float>(rz_p, P.partials, SL_B);
  }
  if (!P.resume) {
  if (!grid_reduce_sync_wide(P.bar, P.st, P.limit_ns, P.partials, P.totals, 0, 2 * NR)) return;
  if (threadIdx.x < NR) {
    const int c = threadIdx.x;
    s_bnorm[c] = sqrt(__ldcg(P.totals + SL_A + c));
    s_rz[c] = __ldcg(P.totals + SL_B + c);
    s_rmax[c] = s_bnorm[c];
    s_res[c] = s_bnorm[c];
    s_active[c] = s_bnorm[c] >= 1e-30;
    s_citers[c] = 0;
    s_restart[c] = 0;
    s_rrec[c] = s_bnorm[c];
    if (!s_active[c]) s_res[c] = 0.0;
  }
  __syncthreads();
  if constexpr (COARSE) {  // P = D^-1 B + Z M Z^T B
    if (!coarse_step_m(P, gwarp, nwarps, lane, ring)) return;
    if (threadIdx.x < NR) s_rz[threadIdx.x] += __ldcg(P.totals + SL_A + threadIdx.x);
    for (long long q = tid; q < nq; q += nth) {
      float p[CPL], zc[CPL];
      ld4(P.P32 + q * CPL, p);
      coarse_prolong_m(P.C, q / LPG, CPL * (int)(q % LPG), zc);
#pragma unroll
      for (int c = 0; c < CPL; ++c) p[c] += zc[c];
      st4(P.P32 + q * CPL, p);
    }
    if (!grid_sync(P.bar, P.st, P.limit_ns)) return;
  }
  }
  long long iters = iters0;
  int updates = updates0, status = AXIA_OK;
  for (long long it = it0; it < P.max_iter; ++it) {
    int any = 0;
    for (int c = 0; c < NR; ++c) any |= s_active[c];
    if (!any) break;
    iters = it + 1;
    // Q = K P (FP32) and per-column p.q
    float pq_p[TC];
#pragma unroll
    for (int c = 0; c < TC; ++c) pq_p[c] = 0.f;
    RowStage* const stg = s_stage + 2 * (threadIdx.x >> 5);
    stage_row(gwarp, lane, P.M32, stg);
    int kb = 0;
    for (int a = gwarp; a < n_nodes; a += nwarps, kb ^= 1) {
      stage_row(a + nwarps, lane, P.M32, stg + (kb ^ 1));
      cp_async_wait<1>();  // this row's copies (all but the group just opened)
      __syncwarp();
      float y[3][TC];
      const int len = __ldg(P.M32.adj_ptr + a + 1) - __ldg(P.M32.adj_ptr + a);
      if (len <= STAGE_B)
        row_tile<TC, TU, true>(a, len, lane, stg + kb, P.M32, P.P32, y);
      else
        row_tile<TC, TU, false>(a, len, lane, stg + kb, P.M32, P.P32, y);
      __syncwarp();  // every lane is done with stg[kb] before it is refilled
      if (lane < NR / TC) {
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const size_t off = (size_t)(3 * a + i) * NR + TC * lane;
          float p[TC];
          ldc<TC>(P.P32 + off, p);
          stc<TC>(P.Q32 + off, y[i]);
#pragma unroll
          for (int c = 0; c < TC; ++c) pq_p[c] = fmaf(p[c], y[i][c], pq_p[c]);
        }
      }
    }
    cp_async_wait<0>();  // the last (empty or unused) group
    // lanes 0 .. 32/TC - 1 hold the columns TC lane .. TC lane + TC - 1 of their warp
    block_partials_cols<float, TC>(pq_p, P.partials, SL_A);
    if (!grid_reduce_sync_wide(P.bar, P.st, P.limit_ns, P.partials, P.totals, SL_A, NR)) return;
    if (threadIdx.x < NR) {
      const int c = threadIdx.x;
      const double pq = __ldcg(P.totals + SL_A + c);
      float al = 0.f;
      if (s_active[c]) {
        if (!(fabs(pq) >= 1e-30) || !isfinite(pq)) {
          s_active[c] = 0;  // breakdown: freeze the column, report below
          s_res[c] = -1.0;
        } else {
          al = (float)(s_rz[c] / pq);
          s_citers[c] = it + 1;
        }
      }
      s_alpha[c] = al;
    }
    __syncthreads();
    float rr_p[CPL] = {0, 0, 0, 0}, rzn_p[CPL] = {0, 0, 0, 0};
    for (long long q = tid; q < nq; q += nth) {
      const long long row = q / LPG;
      const int c0 = CPL * (int)(q % LPG);
      float x[CPL], r[CPL], p[CPL], qq[CPL];
      ld4(P.X32 + q * CPL, x);
      ld4(P.R32 + q * CPL, r);
      ld4(P.P32 + q * CPL, p);
      ld4(P.Q32 + q * CPL, qq);
      const float di = P.dinv32[row];
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        const float al = s_alpha[c0 + c];
        x[c] = fmaf(al, p[c], x[c]);
        r[c] = fmaf(-al, qq[c], r[c]);
        rr_p[c] = fmaf(r[c], r[c], rr_p[c]);
        rzn_p[c] = fmaf(r[c], r[c] * di, rzn_p[c]);
      }
      st4(P.X32 + q * CPL, x);
      st4(P.R32 + q * CPL, r);
    }
    block_partials_cols<float>(rr_p, P.partials, SL_A);
    __syncthreads();
    block_partials_cols<float>(rzn_p, P.partials, SL_B);
    if (!grid_reduce_sync_wide(P.bar, P.st, P.limit_ns, P.partials, P.totals, 0, 2 * NR)) return;
    if (threadIdx.x == 0) {
      int all_dropped = 1, candidate = 0, seen = 0;
      for (int c = 0; c < NR; ++c) {
        if (!s_active[c]) continue;
        seen = 1;
        const double rn = sqrt(__ldcg(P.totals + SL_A + c));
        s_rrec[c] = rn;
        if (!isfinite(rn)) candidate = 1;
        if (rn > P.delta * s_rmax[c]) all_dropped = 0;
        if (rn <= P.tol * s_bnorm[c]) candidate = 1;
      }
      s_flag = seen && (all_dropped || candidate);
    }
    __syncthreads();
    if (s_flag && P.split) {  // the update runs as its own launches; resume from the state
      if (blockIdx.x == 0) {
        if (threadIdx.x < NR) {
          const int c = threadIdx.x;
          P.state->rz[c] = s_rz[c];
          P.state->bnorm[c] = s_bnorm[c];
          P.state->rmax[c] = s_rmax[c];
          P.state->res[c] = s_res[c];
          P.state->active[c] = s_active[c];
          P.state->citers[c] = s_citers[c];
          P.state->rrec[c] = s_rrec[c];
        }
        if (threadIdx.x == 0) {
          P.state->it = it;
          P.state->iters = iters;
          P.state->updates = updates;
          P.state->phase = 1;
        }
      }
      return;
    }
    if (s_flag) {
      // reliable update for all columns: x += x32, r = b - K x (FP64), r32 = r
      for (long long q = tid; q < nq; q += nth) {
        double x[CPL];
        float x32[CPL];
        const float fz4[CPL] = {0, 0, 0, 0};
        ld4(P.X + q * CPL, x);
        ld4(P.X32 + q * CPL, x32);
#pragma unroll
        for (int c = 0; c < CPL; ++c) x[c] += (double)x32[c];
        st4(P.X + q * CPL, x);
        st4(P.X32 + q * CPL, fz4);
      }
      if (!grid_sync(P.bar, P.st, P.limit_ns)) return;
      double rr64[CPL] = {0, 0, 0, 0};
      float rz2[CPL] = {0, 0, 0, 0};
      for (int a = gwarp; a < n_nodes; a += nwarps) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          double y[3][2];
          bsr_row_multi_half(a, lane, P.M64, P.X, h, y);
          if (lane < LPG) {
#pragma unroll
            for (int i = 0; i < 3; ++i) {
              const size_t off = (size_t)(3 * a + i) * NR + CPL * lane + 2 * h;
              const double2 bv = *reinterpret_cast<const double2*>(P.B + off);
              const float di = P.dinv32[3 * a + i];
              const double rv0 = bv.x - y[i][0], rv1 = bv.y - y[i][1];
              rr64[2 * h] = fma(rv0, rv0, rr64[2 * h]);
              rr64[2 * h + 1] = fma(rv1, rv1, rr64[2 * h + 1]);
              const float2 r32 = make_float2((float)rv0, (float)rv1);
              rz2[2 * h] = fmaf(r32.x, r32.x * di, rz2[2 * h]);
              rz2[2 * h + 1] = fmaf(r32.y, r32.y * di, rz2[2 * h + 1]);
              *reinterpret_cast<float2*>(P.R32 + off) = r32;
            }
          }
        }
      }
      block_partials_cols<double>(rr64, P.partials, SL_A);
      __syncthreads();
      block_partials_cols<float>(rz2, P.partials, SL_B);
      if (!grid_reduce_sync_wide(P.bar, P.st, P.limit_ns, P.partials, P.totals, 0, 2 * NR)) return;
      after_update(updates);
    }
    if (!iteration_tail()) return;
  }
  int any_active = 0, broke = 0;
  for (int c = 0; c < NR; ++c) {
    any_active |= s_active[c];
    broke |= s_res[c] < 0.0;
  }
  if (broke) status = AXIA_ERR_ZERO_PIVOT;
  else if (any_active) status = AXIA_ERR_NOT_CONVERGED;
  if (blockIdx.x == 0 && threadIdx.x < NR) {
    const int c = threadIdx.x;
    P.out->bnorm[c] = s_bnorm[c];
    P.out->residual[c] = s_res[c];
    P.out->col_iters[c] = s_citers[c];
    if (c == 0) {
      P.out->iters = iters;
      P.out->updates = updates;
      P.out->status = status;
      if (P.state) P.state->phase = 0;
    }
  }
}

// ---------------------------------------------------------------------------
// Reliable update of the segmented batched solve, as its own launches:
// X += X32 (and X as double words), then R = B - K X with one warp per node
// row and lane c = load case c, then the per-case sums in a fixed order.
// The residual is computed in double words from the FP32 matrix and its low
// parts (K32 + K32lo holds K to 48 bits; FP32-pipe work instead of 9 FP64
// multiply-adds per block and case), or in FP64 from the FP64 matrix.
// ---------------------------------------------------------------------------
__global__ void k_batch_fold(long long n, double* X, float* X32, float* Xh, float* Xl, int split_dw) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const double x = X[t] + f32_to_f64_exact(X32[t]);  // no conversion instruction (FP64 pipe)
    X[t] = x;
    X32[t] = 0.f;
    if (split_dw) {
      const dw xs = dw_split_scaled(x, 0);
      Xh[t] = xs.h;
      Xl[t] = xs.l;
    }
  }
}

template <bool DW>
__global__ void __launch_bounds__(256) k_batch_resid(BsrMatM<float> M32, const float* __restrict__ lo32,
                                                    BsrMatM<double> M64, const double* __restrict__ B,
                                                    const double* __restrict__ X, const float* __restrict__ Xh,
                                                    const float* __restrict__ Xl, const float* __restrict__ dinv32,
                                                    float* R32, double* part, unsigned cases) {
  __shared__ double s_rr[8][NR], s_rz[8][NR];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const bool on = (cases >> lane) & 1u;  // the cases (lanes) this pass computes
  const int n = M32.n_nodes;
  const long long nb = M32.nb;
  double rr = 0.0, rz = 0.0;
  for (int a = blockIdx.x * 8 + w; on && a < n; a += gridDim.x * 8) {
    const int beg = __ldg(M32.adj_ptr + a), end = __ldg(M32.adj_ptr + a + 1);
    double y[3];
    if constexpr (DW) {
      dw_acc acc[3];
      for (int s = beg; s < end; ++s) {
        const int b = __ldg(M32.adj + s);
        dw xv[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const size_t o = (size_t)(3 * b + j) * NR + lane;
          xv[j] = dw{Xh[o], Xl[o]};
        }
#pragma unroll
        for (int p = 0; p < 9; ++p)
          dw_fma(acc[p / 3], dw{__ldg(M32.val + p * nb + s), __ldg(lo32 + p * nb + s)}, xv[p % 3]);
      }
#pragma unroll
      for (int i = 0; i < 3; ++i) y[i] = dw_to_double(dw_value(acc[i]));
    } else {
      y[0] = y[1] = y[2] = 0.0;
      for (int s = beg; s < end; ++s) {
        const int b = __ldg(M64.adj + s);
        double xv[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) xv[j] = X[(size_t)(3 * b + j) * NR + lane];
#pragma unroll
        for (int p = 0; p < 9; ++p) y[p / 3] = fma(__ldg(M64.val + p * nb + s), xv[p % 3], y[p / 3]);
      }
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const size_t o = (size_t)(3 * a + i) * NR + lane;
      const double r = B[o] - y[i];
      rr = fma(r, r, rr);
      const float r32 = (float)r;
      R32[o] = r32;
      rz += (double)(r32 * (r32 * __ldg(dinv32 + 3 * a + i)));
    }
  }
  s_rr[w][lane] = rr;
  s_rz[w][lane] = rz;
  __syncthreads();
  if (w == 0 && on) {  // the other cases keep the partials of an earlier pass
    double a = 0.0, b = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      a += s_rr[k][lane];
      b += s_rz[k][lane];
    }
    part[(size_t)lane * gridDim.x + blockIdx.x] = a;
    part[(size_t)(NR + lane) * gridDim.x + blockIdx.x] = b;
  }
}

// The FP64 residual for a few cases only: KP lanes per node row (the cases
// list[0 .. n-1] on lanes 0 .. n-1 of each group, KP the power of two >= n),
// 32 / KP rows per warp, so the FP64 work follows the number of cases (the
// FP64 pipe charges a warp instruction in full whatever its active lanes).
// Partials of the listed cases only; the others keep an earlier pass's.
struct CaseList {
  int n;
  int c[NR];
};

template <int KP>
__global__ void __launch_bounds__(256) k_batch_resid64_cases(BsrMatM<double> M64, const double* __restrict__ B,
                                                            const double* __restrict__ X,
                                                            const float* __restrict__ dinv32, float* R32,
                                                            double* part, CaseList list) {
  __shared__ double s_rr[8][32], s_rz[8][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int sub = lane % KP, grp = lane / KP;
  constexpr int RPW = 32 / KP;
  const bool on = sub < list.n;
  const int c = on ? list.c[sub] : 0;
  const int n = M64.n_nodes;
  const long long nb = M64.nb;
  double rr = 0.0, rz = 0.0;
  for (int base = (blockIdx.x * 8 + w) * RPW; base < n; base += gridDim.x * 8 * RPW) {
    const int a = base + grp;
    if (!on || a >= n) continue;
    const int beg = __ldg(M64.adj_ptr + a), end = __ldg(M64.adj_ptr + a + 1);
    double y[3] = {0.0, 0.0, 0.0};
    for (int s = beg; s < end; ++s) {
      const int b = __ldg(M64.adj + s);
      double xv[3];
#pragma unroll
      for (int j = 0; j < 3; ++j) xv[j] = X[(size_t)(3 * b + j) * NR + c];
#pragma unroll
      for (int p = 0; p < 9; ++p) y[p / 3] = fma(__ldg(M64.val + p * nb + s), xv[p % 3], y[p / 3]);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const size_t o = (size_t)(3 * a + i) * NR + c;
      const double r = B[o] - y[i];
      rr = fma(r, r, rr);
      const float r32 = (float)r;
      R32[o] = r32;
      rz += (double)(r32 * (r32 * __ldg(dinv32 + 3 * a + i)));
    }
  }
  // the warp's rows of one case: lanes sub, sub + KP, ... (fixed order)
#pragma unroll
  for (int o = KP; o < 32; o <<= 1) {
    rr += __shfl_xor_sync(0xffffffffu, rr, o);
    rz += __shfl_xor_sync(0xffffffffu, rz, o);
  }
  s_rr[w][lane] = rr;
  s_rz[w][lane] = rz;
  __syncthreads();
  if (w == 0 && lane < list.n) {
    double a = 0.0, b = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      a += s_rr[k][lane];
      b += s_rz[k][lane];
    }
    part[(size_t)list.c[lane] * gridDim.x + blockIdx.x] = a;
    part[(size_t)(NR + list.c[lane]) * gridDim.x + blockIdx.x] = b;
  }
}

// totals[k] = sum over the g blocks of part[k][.], ascending block order (one warp per slot)
__global__ void k_batch_resid_sum(const double* part, int g, double* totals) {
  const int lane = threadIdx.x & 31, k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (k >= 2 * NR) return;
  double a = 0.0;
  for (int b = lane; b < g; b += 32) a += part[(size_t)k * g + b];
  a = warp_sum(a);
  if (lane == 0) totals[k] = a;
}

// B[d][c] = f_c[d] - K_fp u0 (free d), 0 (prescribed d); columns >= nrhs zero
__global__ void k_batch_rhs(int64_t nd, int nrhs, const int32_t* ind_of, const double* F, const double* kfu0,
                            double* B) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nd * NR; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t d = t / NR;
    const int c = (int)(t % NR);
    const int r = ind_of[d];
    B[t] = (c < nrhs && r >= 0) ? F[(int64_t)c * nd + d] - kfu0[r] : 0.0;
  }
}
// U_c[d] = u0[d] + X[d][c] on free DOFs
__global__ void k_batch_out(int64_t nd, int nrhs, const int32_t* ind_of, const double* u0, const double* X, double* U) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nd * nrhs; t += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(t / nd);
    const int64_t d = t % nd;
    U[t] = ind_of[d] >= 0 ? u0[d] + X[d * NR + c] : u0[d];
  }
}

// ---------------------------------------------------------------------------
// Block PCG of the 32 load cases (AXIA_BATCH_BLOCK): one Krylov block for all
// cases instead of 32 recurrences.  The breakdown-free form of block CG
// (O'Leary's method with the search block orthonormalized every iteration
// and dependent directions dropped, as in Ji and Li's breakdown-free block
// CG):
//   Q = K P,  Gm = P^T Q,  alpha = Gm^-1 (P^T R),  X += P alpha,  R -= Q alpha,
//   Z = M R,  beta = -Gm^-1 (Q^T Z),  W = Z + P beta,  P = W T  with  P^T P = I
// (T from the Cholesky factor of the scaled W^T W; a direction whose scaled
// pivot falls below 1e-6 is dropped: its column of P is zero).  The 32 x 32
// Gram matrices are reduced in FP64 in a fixed order; alpha, beta and T are
// computed in FP64 and applied to the FP32 blocks.  A load case whose FP64
// residual meets the tolerance is frozen (its alpha column and its column of
// W are zero).  FP64 reliable updates as in the recurrence-per-case kernel.
// No reference counterpart: the reference solves load cases one at a time
// (solver/src/linalg.rs:199-259); the solutions are the same.
// ---------------------------------------------------------------------------
constexpr int BT = 256;             // threads of the block-PCG kernels
constexpr int GRAM_ROWS = 64;       // rows staged per Gram tile
constexpr int NG_MAX = 3;           // Gram products per pass

// Q = K P on [nd][32] blocks: warp per block row, two cases per lane, four
// blocks per group and step
__global__ void __launch_bounds__(BT) k_blk_spmm(BsrMatM<float> M, const float* P, float* Q) {
  const int lane = threadIdx.x & 31;
  const int gwarp = (blockIdx.x * BT + threadIdx.x) >> 5, nwarps = (gridDim.x * BT) >> 5;
  for (int a = gwarp; a < M.n_nodes; a += nwarps) {
    const int len = __ldg(M.adj_ptr + a + 1) - __ldg(M.adj_ptr + a);
    float y[3][2];
    row_tile<2, 4, false>(a, len, lane, nullptr, M, P, y);
    if (lane < 16) {
#pragma unroll
      for (int i = 0; i < 3; ++i) stc<2>(Q + (size_t)(3 * a + i) * NR + 2 * lane, y[i]);
    }
  }
}

// Gram products G_g = A^T B_g (g < ng) over the rows of [nd][32] blocks; a block
// takes tiles of GRAM_ROWS rows in turn (staged in shared memory), thread t owns
// entries (t / 8, 4 (t % 8) .. + 3) of each product, sums a tile in FP32 and
// the tiles in FP64, and writes its 32 x 32 partials to part[block][g].
__global__ void __launch_bounds__(BT) k_blk_gram(int64_t nd, const float* A, const float* B0, const float* B1,
                                                 const float* B2, int ng, double* part) {
  __shared__ __align__(16) float sA[GRAM_ROWS][NR];
  __shared__ __align__(16) float sB[NG_MAX][GRAM_ROWS][NR];
  const float* Bs[NG_MAX] = {B0, B1, B2};
  const int i = threadIdx.x >> 3, j4 = 4 * (threadIdx.x & 7);
  double acc[NG_MAX][4] = {};
  const int64_t ntile = (nd + GRAM_ROWS - 1) / GRAM_ROWS;
  for (int64_t tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
    const int64_t r0 = tile * GRAM_ROWS;
    const int rows = nd - r0 < GRAM_ROWS ? (int)(nd - r0) : GRAM_ROWS;
    __syncthreads();
    for (int t = threadIdx.x; t < GRAM_ROWS * NR / 4; t += BT) {
      const int r = t / (NR / 4), c = 4 * (t % (NR / 4));
      const bool ok = r < rows;
      const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
      *reinterpret_cast<float4*>(&sA[r][c]) = ok ? __ldcs(reinterpret_cast<const float4*>(A + (r0 + r) * NR + c)) : z;
#pragma unroll
      for (int g = 0; g < NG_MAX; ++g)
        if (g < ng)
          *reinterpret_cast<float4*>(&sB[g][r][c]) =
              ok ? __ldcs(reinterpret_cast<const float4*>(Bs[g] + (r0 + r) * NR + c)) : z;
    }
    __syncthreads();
#pragma unroll
    for (int g = 0; g < NG_MAX; ++g) {
      if (g >= ng) break;
      float s[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 8
      for (int r = 0; r < GRAM_ROWS; ++r) {
        const float a = sA[r][i];
        const float4 b = *reinterpret_cast<const float4*>(&sB[g][r][j4]);
        s[0] = fmaf(a, b.x, s[0]);
        s[1] = fmaf(a, b.y, s[1]);
        s[2] = fmaf(a, b.z, s[2]);
        s[3] = fmaf(a, b.w, s[3]);
      }
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[g][c] += (double)s[c];
    }
  }
#pragma unroll
  for (int g = 0; g < NG_MAX; ++g)
    if (g < ng)
#pragma unroll
      for (int c = 0; c < 4; ++c) part[((size_t)blockIdx.x * NG_MAX + g) * NR * NR + i * NR + j4 + c] = acc[g][c];
}

// out[e] = sum over blocks b of part[b][src + e], e < n_entries (part rows of
// NG_MAX * 1024 doubles): 16 threads per entry take every 16th block and
// their sums are added in a fixed pattern, so the result is reproducible
__global__ void __launch_bounds__(BT) k_blk_finalize(int nblk, int src, int n_entries, const double* part,
                                                     double* out) {
  const int t = blockIdx.x * BT + threadIdx.x;
  const int e = t >> 4, k = t & 15;
  double s = 0.0;
  if (e < n_entries)
    for (int b = k; b < nblk; b += 16) s += __ldcg(part + (size_t)b * NG_MAX * NR * NR + src + e);
#pragma unroll
  for (int o = 1; o < 16; o <<= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (e < n_entries && k == 0) out[e] = s;
}

// Out = (acc ? Out : 0) + sgn In M over the rows (M 32 x 32 FP32); columns
// whose bit of `zero_cols` is set come out zero.  With `norms`, each block
// also writes the sums of squares of its output rows per column to
// part[block][3][..] (the fourth slot of the Gram partials).
__global__ void __launch_bounds__(BT, 4) k_blk_mm(int64_t nd, const float* In, const float* Mx, float sgn, int acc,
                                               unsigned zero_cols, float* Out, double* norm_part) {
  __shared__ __align__(16) float sM[NR][NR];
  __shared__ double sN[BT / 8][NR];
  for (int t = threadIdx.x; t < NR * NR; t += BT) sM[t / NR][t % NR] = Mx[t];
  __syncthreads();
  const int j4 = 4 * (threadIdx.x & 7);
  double nrm[4] = {0.0, 0.0, 0.0, 0.0};
  for (int64_t r = (int64_t)blockIdx.x * (BT / 8) + (threadIdx.x >> 3); r < nd; r += (int64_t)gridDim.x * (BT / 8)) {
    const float4* in = reinterpret_cast<const float4*>(In + r * NR);
    float o[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 4
    for (int q = 0; q < 8; ++q) {
      const float4 v = in[q];
      const float vk[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const float4 m = *reinterpret_cast<const float4*>(&sM[4 * q + u][j4]);
        o[0] = fmaf(vk[u], m.x, o[0]);
        o[1] = fmaf(vk[u], m.y, o[1]);
        o[2] = fmaf(vk[u], m.z, o[2]);
        o[3] = fmaf(vk[u], m.w, o[3]);
      }
    }
    float4* out = reinterpret_cast<float4*>(Out + r * NR + j4);
    const float4 prev = acc ? *out : make_float4(0.f, 0.f, 0.f, 0.f);
    float res[4] = {fmaf(sgn, o[0], prev.x), fmaf(sgn, o[1], prev.y), fmaf(sgn, o[2], prev.z), fmaf(sgn, o[3], prev.w)};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      if ((zero_cols >> (j4 + c)) & 1u) res[c] = 0.f;
      nrm[c] = fma((double)res[c], (double)res[c], nrm[c]);
    }
    *out = make_float4(res[0], res[1], res[2], res[3]);
  }
  if (norm_part) {
#pragma unroll
    for (int c = 0; c < 4; ++c) sN[threadIdx.x >> 3][j4 + c] = nrm[c];
    __syncthreads();
    if (threadIdx.x < NR) {
      double s = 0.0;
      for (int w = 0; w < BT / 8; ++w) s += sN[w][threadIdx.x];
      norm_part[((size_t)blockIdx.x * NG_MAX) * NR * NR + threadIdx.x] = s;
    }
  }
}

// z = D^-1 r (+ the coarse part Z_c y) on [nd][32] blocks, float4 per thread
template <bool COARSE>
__global__ void __launch_bounds__(BT) k_blk_precond(int64_t nd, const float* dinv, const float* R, CoarseArgs C,
                                                    float* Z) {
  const int64_t nq = nd * LPG;
  for (int64_t q = blockIdx.x * (int64_t)BT + threadIdx.x; q < nq; q += (int64_t)gridDim.x * BT) {
    const int64_t row = q / LPG;
    float r[CPL], zc[CPL] = {0.f, 0.f, 0.f, 0.f};
    ld4(R + q * CPL, r);
    if constexpr (COARSE) coarse_prolong_m(C, row, CPL * (int)(q % LPG), zc);
    const float di = dinv[row];
#pragma unroll
    for (int c = 0; c < CPL; ++c) zc[c] = fmaf(r[c], di, zc[c]);
    st4(Z + q * CPL, zc);
  }
}

__global__ void __launch_bounds__(BT) k_blk_restrict(CoarseArgs C, const float* R) {
  const int lane = threadIdx.x & 31;
  const int gwarp = (blockIdx.x * BT + threadIdx.x) >> 5, nwarps = (gridDim.x * BT) >> 5;
  coarse_restrict_m(C, R, gwarp, nwarps, lane);
}

__global__ void __launch_bounds__(PCG_THREADS) k_blk_coarse_solve(CoarseArgs C, double* scratch) {
  extern __shared__ __align__(16) float s_ring[];  // COARSE_RING_FLOATS
  coarse_solve_m(C, s_ring, scratch, 0);
}

// X += X32 (FP64), X32 = 0
__global__ void __launch_bounds__(BT) k_blk_xadd(int64_t n, double* X, float* X32) {
  for (int64_t t = blockIdx.x * (int64_t)BT + threadIdx.x; t < n; t += (int64_t)gridDim.x * BT) {
    X[t] += (double)X32[t];
    X32[t] = 0.f;
  }
}

// R = B - K X in FP64 (lane = load case), R32 = (float) R, per-case sums of
// squares of R to part[block][3][..]
__global__ void __launch_bounds__(BT) k_blk_residual64(BsrMatM<double> M, const double* X, const double* B, float* R32,
                                                       double* norm_part) {
  __shared__ double sN[BT / 32][NR];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gwarp = (blockIdx.x * BT + threadIdx.x) >> 5, nwarps = (gridDim.x * BT) >> 5;
  double nrm = 0.0;
  for (int a = gwarp; a < M.n_nodes; a += nwarps) {
    const int beg = __ldg(M.adj_ptr + a), end = __ldg(M.adj_ptr + a + 1);
    double y0 = 0.0, y1 = 0.0, y2 = 0.0;
    for (int s = beg; s < end; s += 4) {
      double x[4][3], v[4][9];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int su = s + u < end ? s + u : beg;
        const int b = ld_stream(M.adj + su);
#pragma unroll
        for (int j = 0; j < 3; ++j) x[u][j] = s + u < end ? X[(size_t)(3 * b + j) * NR + lane] : 0.0;
#pragma unroll
        for (int k = 0; k < 9; ++k) v[u][k] = ld_stream(M.val + (long long)k * M.nb + su);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        y0 = fma(v[u][0], x[u][0], fma(v[u][1], x[u][1], fma(v[u][2], x[u][2], y0)));
        y1 = fma(v[u][3], x[u][0], fma(v[u][4], x[u][1], fma(v[u][5], x[u][2], y1)));
        y2 = fma(v[u][6], x[u][0], fma(v[u][7], x[u][1], fma(v[u][8], x[u][2], y2)));
      }
    }
    const double y[3] = {y0, y1, y2};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const size_t off = (size_t)(3 * a + i) * NR + lane;
      const double r = B[off] - y[i];
      nrm = fma(r, r, nrm);
      R32[off] = (float)r;
    }
  }
  sN[warp][lane] = nrm;
  __syncthreads();
  if (threadIdx.x < NR) {
    double s = 0.0;
    for (int w = 0; w < BT / 32; ++w) s += sN[w][threadIdx.x];
    norm_part[((size_t)blockIdx.x * NG_MAX) * NR * NR + threadIdx.x] = s;
  }
}

// The small dense steps (one block of 32 x 32 threads, FP64, thread (r, c)
// owns entry (r, c); every elimination step is one synchronised parallel
// update, so a step costs a barrier instead of a serial loop):
//   mode 0 (alpha): G = Gram 0 (P^T Q, kept as Gm), S = Gram 1 (P^T R):
//           alpha = Gm^-1 S, zero in the columns of `frozen`
//   mode 1 (beta):  Gm (kept), S = Gram 1 (Q^T Z): beta = -Gm^-1 S
//   mode 2 (orth):  G = Gram 2 (W^T W): T = D L^-T for D G D = L L^T,
//           D = diag(G)^-1/2; a scaled pivot below 1e-6 (or a zero column)
//           drops that direction (its row and column of T are zero)
// gram: [4][32][32] (Gm, S, WtW, norms); small: [3][32][32] FP32 alpha, beta, T.
// Gm's factor is recomputed each time (a 32 x 32 Cholesky is a few microseconds).
__global__ void __launch_bounds__(NR * NR) k_blk_small(int mode, unsigned frozen, const double* gram, float* small) {
  __shared__ double L[NR][NR + 1];
  __shared__ double S[NR][NR + 1];
  __shared__ double dsc[NR];
  __shared__ int drop[NR];
  __shared__ double s_thr;
  const int r = threadIdx.x / NR, c = threadIdx.x % NR;
  const double* G = gram + (mode == 2 ? 2 : 0) * NR * NR;
  if (r == 0) {
    const double gd = G[c * NR + c];
    dsc[c] = mode != 2 ? 1.0 : (gd > 1e-300 ? 1.0 / sqrt(gd) : 0.0);
  }
  __syncthreads();
  L[r][c] = G[r * NR + c] * dsc[r] * dsc[c];
  S[r][c] = mode == 2 ? (r == c ? 1.0 : 0.0) : gram[NR * NR + r * NR + c];
  __syncthreads();
  if (threadIdx.x == 0) {
    double dmax = 0.0;
    for (int i = 0; i < NR; ++i) dmax = fmax(dmax, L[i][i]);
    s_thr = mode == 2 ? 1e-6 : 1e-12 * dmax;
  }
  __syncthreads();
  // right-looking Cholesky L L^T in the lower triangle; a dropped pivot gets a
  // unit diagonal and a zero column, so it drops out of the later steps
  for (int k = 0; k < NR; ++k) {
    if (threadIdx.x == 0) {
      const double piv = L[k][k];
      const int dr = !(piv > s_thr) || (mode == 2 && dsc[k] == 0.0);
      drop[k] = dr;
      L[k][k] = dr ? 1.0 : sqrt(piv);
    }
    __syncthreads();
    if (c == 0 && r > k) L[r][k] = drop[k] ? 0.0 : L[r][k] / L[k][k];
    __syncthreads();
    if (r > k && c > k && c <= r) L[r][c] -= L[r][k] * L[c][k];
    __syncthreads();
  }
  if (mode != 2) {
    // forward substitution L y = S (every column c of S at once)
    for (int i = 0; i < NR; ++i) {
      if (r == i) S[i][c] = drop[i] ? 0.0 : S[i][c] / L[i][i];
      __syncthreads();
      if (r > i) S[r][c] -= L[r][i] * S[i][c];
      __syncthreads();
    }
  }
  // backward substitution L^T x = y (mode 2: x = L^-T from S = I)
  for (int i = NR - 1; i >= 0; --i) {
    if (r == i) S[i][c] = drop[i] ? 0.0 : S[i][c] / L[i][i];
    __syncthreads();
    if (r < i) S[r][c] -= L[i][r] * S[i][c];
    __syncthreads();
  }
  double v;
  if (mode == 2)
    v = (drop[r] || drop[c]) ? 0.0 : dsc[r] * S[r][c];
  else if (mode == 0)
    v = ((frozen >> c) & 1u) ? 0.0 : S[r][c];
  else
    v = -S[r][c];
  small[mode * NR * NR + r * NR + c] = (float)v;
}

// R32 = (float) B, X = 0, X32 = 0, per-case sums of squares of B to part[block][0][..]
__global__ void __launch_bounds__(BT) k_blk_init(int64_t n, const double* B, double* X, float* X32, float* R32,
                                                 double* norm_part) {
  __shared__ double sN[BT / 32][NR];
  double nrm = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)BT + threadIdx.x; t < n; t += (int64_t)gridDim.x * BT) {
    const double b = B[t];
    X[t] = 0.0;
    X32[t] = 0.f;
    R32[t] = (float)b;
    nrm = fma(b, b, nrm);  // this thread's case: t % 32 = lane
  }
  sN[threadIdx.x >> 5][threadIdx.x & 31] = nrm;
  __syncthreads();
  if (threadIdx.x < NR) {
    double s = 0.0;
    for (int w = 0; w < BT / 32; ++w) s += sN[w][threadIdx.x];
    norm_part[((size_t)blockIdx.x * NG_MAX) * NR * NR + threadIdx.x] = s;
  }
}

// Tile shapes the batched kernel is instantiated for: (load cases per lane,
// blocks per group and step).
struct BatchTile {
  int tc, tu;
};
// ((4, 2) is left out: it spills about 100 bytes of registers with the coarse space.)
constexpr BatchTile kBatchTiles[] = {{4, 1}, {2, 2}, {2, 4}, {1, 4}, {1, 8}};
constexpr BatchTile kBatchDefault = {2, 4};

template <bool COARSE>
const void* batch_kernel(BatchTile t) {
  switch (t.tc * 100 + t.tu) {
    case 401: return (const void*)pcg_bsr_multi_kernel<COARSE, 4, 1>;
    case 202: return (const void*)pcg_bsr_multi_kernel<COARSE, 2, 2>;
    case 204: return (const void*)pcg_bsr_multi_kernel<COARSE, 2, 4>;
    case 104: return (const void*)pcg_bsr_multi_kernel<COARSE, 1, 4>;
    case 108: return (const void*)pcg_bsr_multi_kernel<COARSE, 1, 8>;
    default: return nullptr;
  }
}

bool valid_tile(int tc, int tu) {
  for (const BatchTile& t : kBatchTiles)
    if (t.tc == tc && t.tu == tu) return true;
  return false;
}

int ensure_batch_buffers(axia_ctx* ctx) {
  const size_t blk = (size_t)ctx->ndof * NR;
  if (ctx->batch_capacity < blk) {
    AXIA_TRY(dev_alloc(ctx, &ctx->d_mB, blk));
    AXIA_TRY(dev_alloc(ctx, &ctx->d_mX, blk));
    AXIA_TRY(dev_alloc(ctx, &ctx->d_mX32, blk));
    AXIA_TRY(dev_alloc(ctx, &ctx->d_mR32, blk));
    AXIA_TRY(dev_alloc(ctx, &ctx->d_mP32, blk));
    AXIA_TRY(dev_alloc(ctx, &ctx->d_mQ32, blk));
    ctx->batch_capacity = blk;
  }
  if (!ctx->d_mout) {
    MultiOut* o = nullptr;
    AXIA_TRY(dev_alloc(ctx, &o, 1));
    ctx->d_mout = o;
  }
  return AXIA_OK;
}

// Grid of the cooperative launch of kern (its occupancy with the staging buffers).
int batch_grid(axia_ctx* ctx, const void* kern, int* grid) {
  // static + staging shared memory is above the 48 KB a block gets without opting in
  AXIA_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)DYN_BYTES));
  AXIA_TRY(coop_grid(ctx, kern, (int)std::min<int64_t>(ctx->ndof, INT32_MAX), grid, DYN_BYTES));
  if ((size_t)*grid * 2 * NR > ctx->partial_slots) *grid = (int)(ctx->partial_slots / (2 * NR));
  return AXIA_OK;
}

MultiArgs multi_args(axia_ctx* ctx, double rtol, double delta, long long max_iter, const CoarseArgs& cargs) {
  return MultiArgs{BsrMatM<float>{(int)ctx->n_nodes, ctx->d_qptr, ctx->d_qadj, ctx->d_bval32, (long long)ctx->nbq},
                   BsrMatM<double>{(int)ctx->n_nodes, ctx->d_qptr, ctx->d_qadj, ctx->d_bval64, (long long)ctx->nbq},
                   (int)ctx->ndof, ctx->d_bdinv32, ctx->d_mB, ctx->d_mX, ctx->d_mX32, ctx->d_mR32, ctx->d_mP32,
                   ctx->d_mQ32, ctx->d_partials, ctx->d_totals, ctx->d_bar, ctx->d_status, (MultiOut*)ctx->d_mout,
                   rtol, delta, max_iter, 2000000000ull, cargs};
}

int launch_batch(axia_ctx* ctx, const void* kern, int grid, MultiArgs& P) {
  void* params[] = {&P};
  AXIA_CUDA(ctx, cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(PCG_THREADS), params, DYN_BYTES, ctx->stream));
  ctx->launches++;
  return AXIA_OK;
}

// B[d][c] = (1 + c / 32) on free DOFs: the autotuner's load (every column busy)
__global__ void k_batch_tune_rhs(int64_t nd, const int32_t* ind_of, double* B) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nd * NR; t += (int64_t)gridDim.x * blockDim.x)
    B[t] = ind_of[t / NR] >= 0 ? 1.0 + (double)(t % NR) / NR : 0.0;
}

std::string batch_tune_key(const axia_ctx* ctx) {
  cudaDeviceProp prop{};
  cudaGetDeviceProperties(&prop, ctx->device);
  const double rb = ctx->n_nodes ? (double)ctx->nbq / (double)ctx->n_nodes : 0.0;
  int bucket = 0;
  for (int64_t n = ctx->n_nodes; n > 1; n >>= 1) ++bucket;
  std::string name(prop.name);
  for (char& c : name)
    if (c == '"' || c == '\\') c = '_';
  return name + "|batch32|nn=" + std::to_string(ctx->nn) + "|r=" + std::to_string(ctx->reduced) +
         "|rowblocks=" + std::to_string((int)std::lround(rb)) + "|log2nodes=" + std::to_string(bucket);
}

bool batch_cache_lookup(const char* path, const std::string& key, int* tc, int* tu) {
  FILE* fh = path ? std::fopen(path, "r") : nullptr;
  if (!fh) return false;
  char line[1024];
  const std::string want = "\"key\": \"" + key + "\"";
  bool found = false;
  while (std::fgets(line, sizeof(line), fh)) {
    const std::string l(line);
    if (l.find(want) == std::string::npos) continue;
    const size_t pc = l.find("\"cases_per_lane\": "), pu = l.find("\"blocks_per_step\": ");
    if (pc == std::string::npos || pu == std::string::npos) continue;
    *tc = std::atoi(l.c_str() + pc + 18);
    *tu = std::atoi(l.c_str() + pu + 19);
    found = true;  // the last matching line wins
  }
  std::fclose(fh);
  return found;
}

}  // namespace

// Autotuner of the batched kernel's tile: every instantiated (cases per lane,
// blocks per step) pair runs 30 CG iterations of the 32-case solve (diagonal
// preconditioner, a load on every free DOF of every case), timed with CUDA
// events on the context's stream (best of two); the fastest per iteration is
// kept for later batched solves and appended to the JSON-lines cache.
int batch_autotune(axia_ctx* ctx, const char* cache_path, int* tc_out, int* tu_out, double* us_out) {
  if (!ctx->have_bsr64 || !ctx->have_bsr32)
    return set_error(ctx, AXIA_ERR_STATE, "batch autotune needs the node-block forms (AXIA_ASM_BSR64 | AXIA_ASM_BSR32)");
  const std::string key = batch_tune_key(ctx);
  int tc = 0, tu = 0;
  if (batch_cache_lookup(cache_path, key, &tc, &tu) && valid_tile(tc, tu)) {
    ctx->tuned_btc = tc;
    ctx->tuned_btu = tu;
    *tc_out = tc;
    *tu_out = tu;
    if (us_out) *us_out = 0.0;
    return AXIA_OK;
  }
  AXIA_TRY(ensure_batch_buffers(ctx));
  k_batch_tune_rhs<<<ctx->sm_count * 8, 256, 0, ctx->stream>>>(ctx->ndof, ctx->d_ind_of, ctx->d_mB);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  const long long iters = 30;
  double best = 1e300;
  BatchTile pick = kBatchDefault;
  cudaEvent_t a = nullptr, b = nullptr;
  int st = AXIA_OK;
  if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess)
    st = set_error(ctx, AXIA_ERR_CUDA, "batch autotune events");
  for (const BatchTile& t : kBatchTiles) {
    if (st != AXIA_OK) break;
    const void* kern = batch_kernel<false>(t);
    int grid = 0;
    if ((st = batch_grid(ctx, kern, &grid)) != AXIA_OK) break;
    float best_t = 1e30f;
    for (int rep = 0; rep < 2 && st == AXIA_OK; ++rep) {
      if ((st = reset_dev_status(ctx)) != AXIA_OK) break;
      cudaMemsetAsync(ctx->d_bar, 0, sizeof(GridBarrier), ctx->stream);
      MultiArgs P = multi_args(ctx, 1e-30, 1e-30, iters, CoarseArgs{});
      cudaEventRecord(a, ctx->stream);
      if ((st = launch_batch(ctx, kern, grid, P)) != AXIA_OK) break;
      cudaEventRecord(b, ctx->stream);
      MultiOut o;
      if (cudaMemcpyAsync(&o, ctx->d_mout, sizeof(MultiOut), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
          cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        st = set_error(ctx, AXIA_ERR_CUDA, "batch autotune launch");
        break;
      }
      DevStatus hs;
      if ((st = read_dev_status(ctx, &hs)) != AXIA_OK) break;
      if (hs.timeout) {
        st = set_error(ctx, AXIA_ERR_TIMEOUT, "a grid barrier of the batched PCG ran past its limit");
        break;
      }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, a, b);
      best_t = std::min(best_t, ms / (float)std::max<long long>(o.iters, 1));
    }
    if (st == AXIA_OK && best_t < best) {
      best = best_t;
      pick = t;
    }
  }
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (st != AXIA_OK) return st;
  ctx->tuned_btc = pick.tc;
  ctx->tuned_btu = pick.tu;
  *tc_out = pick.tc;
  *tu_out = pick.tu;
  if (us_out) *us_out = best * 1e3;
  if (cache_path) {
    if (FILE* fh = std::fopen(cache_path, "a")) {
      std::fprintf(fh, "{\"key\": \"%s\", \"cases_per_lane\": %d, \"blocks_per_step\": %d, \"us_per_iter\": %.3f}\n",
                   key.c_str(), pick.tc, pick.tu, best * 1e3);
      std::fclose(fh);
    }
  }
  return AXIA_OK;
}

namespace {

int ensure_block_buffers(axia_ctx* ctx, int grid) {
  AXIA_TRY(ensure_batch_buffers(ctx));
  if (!ctx->d_mZ32) AXIA_TRY(dev_alloc(ctx, &ctx->d_mZ32, (size_t)ctx->ndof * NR));
  const size_t need = (size_t)grid * NG_MAX * NR * NR;
  if (ctx->bpart_capacity < need) {
    dev_free(ctx->d_bpart);
    ctx->d_bpart = nullptr;
    AXIA_TRY(dev_alloc(ctx, &ctx->d_bpart, need));
    ctx->bpart_capacity = need;
  }
  if (!ctx->d_bgram) AXIA_TRY(dev_alloc(ctx, &ctx->d_bgram, (size_t)4 * NR * NR));
  if (!ctx->d_bsmall) AXIA_TRY(dev_alloc(ctx, &ctx->d_bsmall, (size_t)3 * NR * NR));
  return AXIA_OK;
}

// The launches of one block-PCG solve of 32 cases on ctx->stream.
struct BlockRun {
  axia_ctx* ctx;
  int64_t nd;
  int g_row, g_gram, g_mm;
  CoarseArgs C;
  bool coarse;
  cudaStream_t s;
  double* part() const { return ctx->d_bpart; }
  double* gram(int k) const { return ctx->d_bgram + (size_t)k * NR * NR; }
  float* small(int k) const { return ctx->d_bsmall + (size_t)k * NR * NR; }
  BsrMatM<float> m32() const {
    return BsrMatM<float>{(int)ctx->n_nodes, ctx->d_qptr, ctx->d_qadj, ctx->d_bval32, (long long)ctx->nbq};
  }
  BsrMatM<double> m64() const {
    return BsrMatM<double>{(int)ctx->n_nodes, ctx->d_qptr, ctx->d_qadj, ctx->d_bval64, (long long)ctx->nbq};
  }
  void count(int n) { ctx->launches += n; }
  // Gram products A^T B_g into gram slots dst .. dst + ng - 1
  void gram_pass(const float* A, const float* B0, const float* B1, int ng, int dst) {
    k_blk_gram<<<g_gram, BT, 0, s>>>(nd * 1, A, B0, B1, nullptr, ng, part());
    const int ne = ng * NR * NR;
    k_blk_finalize<<<(ne * 16 + BT - 1) / BT, BT, 0, s>>>(g_gram, 0, ne, part(), gram(dst));
    count(2);
  }
  // the per-case sums of squares written by the last norm kernel (grid nblk) -> gram slot 3
  void norms(int nblk) {
    k_blk_finalize<<<(NR * 16 + BT - 1) / BT, BT, 0, s>>>(nblk, 0, NR, part(), gram(3));
    count(1);
  }
  void mm(const float* In, const float* Mx, float sgn, int acc, unsigned zero_cols, float* Out, bool with_norms) {
    k_blk_mm<<<g_mm, BT, 0, s>>>(nd, In, Mx, sgn, acc, zero_cols, Out, with_norms ? part() : nullptr);
    count(1);
  }
  void small_step(int mode, unsigned frozen) {
    k_blk_small<<<1, NR * NR, 0, s>>>(mode, frozen, ctx->d_bgram, ctx->d_bsmall);
    count(1);
  }
  // Z = M R (diagonal, plus the coarse part)
  void precond(const float* R, float* Z) {
    if (coarse) {
      k_blk_restrict<<<g_row, BT, 0, s>>>(C, R);
      k_blk_coarse_solve<<<ctx->sm_count * 2, PCG_THREADS, COARSE_RING_FLOATS * sizeof(float), s>>>(C, part());
      k_blk_precond<true><<<g_row, BT, 0, s>>>(nd, ctx->d_bdinv32, R, C, Z);
      count(3);
    } else {
      k_blk_precond<false><<<g_row, BT, 0, s>>>(nd, ctx->d_bdinv32, R, C, Z);
      count(1);
    }
  }
  // W = Z (+ P beta), frozen columns zero; T from W^T W; P = W T.  The first
  // time P holds nothing yet: W = Z + 0 (Z beta with the zeroed beta).
  void new_directions(unsigned frozen, bool first) {
    mm(first ? ctx->d_mZ32 : ctx->d_mP32, small(1), first ? 0.f : 1.f, 1, frozen, ctx->d_mZ32, false);
    gram_pass(ctx->d_mZ32, ctx->d_mZ32, nullptr, 1, 2);
    small_step(2, frozen);
    mm(ctx->d_mZ32, small(2), 1.f, 0, 0u, ctx->d_mP32, false);
  }
};

int read_norms(axia_ctx* ctx, double* h) {
  AXIA_CUDA(ctx, cudaMemcpyAsync(h, ctx->d_bgram + 3 * NR * NR, NR * sizeof(double), cudaMemcpyDeviceToHost,
                                 ctx->stream));
  AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return AXIA_OK;
}

}  // namespace

// Block PCG over the load cases (AXIA_KRYLOV_BLOCK), 32 at a time: the launch
// sequence of the breakdown-free block recurrence above, with the per-case
// residual norms read back after every iteration to decide on reliable
// updates, convergence and frozen cases.
int batch_block_solve(axia_ctx* ctx, int nrhs, const double* d_F, double* d_U, const axia_solve_opts* opts,
                      axia_solve_info* info, double* rel_res) {
  if (!ctx->have_bsr64 || !ctx->have_bsr32)
    return set_error(ctx, AXIA_ERR_STATE, "batched solve needs the node-block forms (AXIA_ASM_BSR64 | AXIA_ASM_BSR32)");
  if (opts->preconditioner != AXIA_PRECOND_JACOBI && opts->preconditioner != AXIA_PRECOND_COARSE)
    return set_error(ctx, AXIA_ERR_INVALID_ARG, "batched load cases: unknown preconditioner");
  BlockRun B{};
  B.ctx = ctx;
  B.nd = ctx->ndof;
  B.s = ctx->stream;
  B.g_row = ctx->sm_count * 8;
  B.g_gram = ctx->sm_count * 4;
  B.g_mm = ctx->sm_count * 4;
  B.coarse = opts->preconditioner == AXIA_PRECOND_COARSE;
  AXIA_TRY(ensure_block_buffers(ctx, std::max(B.g_gram, std::max(B.g_mm, B.g_row))));
  if (B.coarse) AXIA_TRY(coarse_prepare_batched(ctx, opts->coarse_nodes, &B.C));
  const long long max_iter = opts->max_iter > 0 ? opts->max_iter : std::max<long long>(4LL * ctx->n_free, 200);
  const double delta = opts->inner_rtol > 0 && opts->inner_rtol < 1 ? opts->inner_rtol : 0.01;
  const double tol = opts->rtol;
  info->iters = 0;
  info->outer_iters = 0;
  double worst = 0.0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  AXIA_CUDA(ctx, cudaEventCreate(&ev0));
  AXIA_CUDA(ctx, cudaEventCreate(&ev1));
  int st = AXIA_OK;
  const int64_t n = B.nd * NR;
  for (int c0 = 0; c0 < nrhs && st == AXIA_OK; c0 += NR) {
    const int nc = std::min(NR, nrhs - c0);
    k_batch_rhs<<<ctx->sm_count * 8, 256, 0, B.s>>>(B.nd, nc, ctx->d_ind_of, d_F + (int64_t)c0 * B.nd, ctx->d_kfu0,
                                                   ctx->d_mB);
    cudaEventRecord(ev0, B.s);
    k_blk_init<<<B.g_row, BT, 0, B.s>>>(n, ctx->d_mB, ctx->d_mX, ctx->d_mX32, ctx->d_mR32, B.part());
    B.count(2);
    B.norms(B.g_row);
    double h[NR], bnorm[NR], rmax[NR], res[NR];
    if ((st = read_norms(ctx, h)) != AXIA_OK) break;
    unsigned frozen = 0u;
    for (int c = 0; c < NR; ++c) {
      bnorm[c] = std::sqrt(h[c]);
      rmax[c] = res[c] = bnorm[c];
      if (!(bnorm[c] >= 1e-30)) {
        frozen |= 1u << c;
        res[c] = 0.0;
      }
    }
    long long iters = 0;
    int updates = 0;
    if (frozen != 0xffffffffu) {
      AXIA_CUDA(ctx, cudaMemsetAsync(B.small(1), 0, NR * NR * sizeof(float), B.s));
      B.precond(ctx->d_mR32, ctx->d_mZ32);
      B.new_directions(frozen, true);
    }
    for (long long it = 0; frozen != 0xffffffffu && it < max_iter; ++it) {
      iters = it + 1;
      // Q = K P; Gm = P^T Q, S = P^T R; alpha = Gm^-1 S; X += P alpha, R -= Q alpha
      k_blk_spmm<<<B.g_row, BT, 0, B.s>>>(B.m32(), ctx->d_mP32, ctx->d_mQ32);
      B.count(1);
      B.gram_pass(ctx->d_mP32, ctx->d_mQ32, ctx->d_mR32, 2, 0);
      B.small_step(0, frozen);
      B.mm(ctx->d_mP32, B.small(0), 1.f, 1, 0u, ctx->d_mX32, false);
      B.mm(ctx->d_mQ32, B.small(0), -1.f, 1, 0u, ctx->d_mR32, true);
      B.norms(B.g_mm);
      if ((st = read_norms(ctx, h)) != AXIA_OK) break;
      bool all_dropped = true, candidate = false;
      for (int c = 0; c < NR; ++c) {
        if ((frozen >> c) & 1u) continue;
        const double rn = std::sqrt(h[c]);
        if (!std::isfinite(rn)) candidate = true;
        if (rn > delta * rmax[c]) all_dropped = false;
        if (rn <= tol * bnorm[c]) candidate = true;
      }
      if (all_dropped || candidate) {
        // reliable update: X += X32, R = B - K X in FP64 for every case
        k_blk_xadd<<<B.g_row, BT, 0, B.s>>>(n, ctx->d_mX, ctx->d_mX32);
        k_blk_residual64<<<B.g_row, BT, 0, B.s>>>(B.m64(), ctx->d_mX, ctx->d_mB, ctx->d_mR32, B.part());
        B.count(2);
        B.norms(B.g_row);
        if ((st = read_norms(ctx, h)) != AXIA_OK) break;
        ++updates;
        for (int c = 0; c < NR; ++c) {
          if ((frozen >> c) & 1u) continue;
          const double rn = std::sqrt(h[c]);
          if (!std::isfinite(rn)) {
            st = set_error(ctx, AXIA_ERR_NONFINITE, "block CG: non-finite residual");
            break;
          }
          res[c] = rmax[c] = rn;
          if (rn <= tol * bnorm[c]) frozen |= 1u << c;
        }
        if (st != AXIA_OK || frozen == 0xffffffffu) break;
      }
      // Z = M R; beta = -Gm^-1 (Q^T Z); W = Z + P beta; P = orth(W)
      B.precond(ctx->d_mR32, ctx->d_mZ32);
      B.gram_pass(ctx->d_mQ32, ctx->d_mZ32, nullptr, 1, 1);
      B.small_step(1, frozen);
      B.new_directions(frozen, false);
    }
    cudaEventRecord(ev1, B.s);
    AXIA_CUDA(ctx, cudaEventSynchronize(ev1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev0, ev1);
    info->ms_pcg_kernel += ms;
    info->pcg_launches += 1;
    if (st != AXIA_OK) break;
    info->iters = std::max<int64_t>(info->iters, iters);
    info->outer_iters += updates;
    for (int c = 0; c < nc; ++c) {
      const double rr = bnorm[c] > 0 ? res[c] / bnorm[c] : 0.0;
      if (rel_res) rel_res[c0 + c] = rr;
      worst = std::max(worst, rr);
    }
    if (frozen != 0xffffffffu) {
      st = set_error(ctx, AXIA_ERR_NOT_CONVERGED, "block CG did not converge in " + std::to_string(iters) + " iterations");
      break;
    }
    k_batch_out<<<ctx->sm_count * 8, 256, 0, B.s>>>(B.nd, nc, ctx->d_ind_of, ctx->d_u0, ctx->d_mX,
                                                   d_U + (int64_t)c0 * B.nd);
    ctx->launches++;
    if (cudaGetLastError() != cudaSuccess) st = set_error(ctx, AXIA_ERR_CUDA, "block CG launch");
  }
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  if (st != AXIA_OK) return st;
  info->residual = worst;
  info->bnorm = 1.0;
  return AXIA_OK;
}

// Solves nrhs load cases (F, U: [nrhs][nd] device arrays) 32 at a time.
int ensure_segment_buffers(axia_ctx* ctx) {
  const size_t blk = (size_t)ctx->ndof * NR;
  if (ctx->seg_capacity < blk) {
    AXIA_TRY(dev_alloc(ctx, &ctx->d_mXh, blk));
    AXIA_TRY(dev_alloc(ctx, &ctx->d_mXl, blk));
    ctx->seg_capacity = blk;
  }
  if (!ctx->d_mstate) {
    BatchState* st = nullptr;
    AXIA_CUDA(ctx, cudaMalloc(&st, sizeof(BatchState)));
    ctx->d_mstate = st;
  }
  return AXIA_OK;
}

// The batched kernel in segments: it stops at each reliable update (phase 1);
// X is folded and R = B - K X computed in double words, then in FP64 for the
// cases whose double-word residual meets its tolerance (the FP64 one decides
// convergence) or has not dropped below half of its previous update's.  If the two residuals of a case then differ by more than 10 %,
// the double-word error floor (about 2^-47 sum |K| |X|) is reached and the
// updates are FP64 from then on.  Then the kernel resumes (phase 0 when it
// finishes).
int run_segmented(axia_ctx* ctx, const void* kern, int grid, MultiArgs& P) {
  const int64_t nd = ctx->ndof;
  const long long n = (long long)nd * NR;
  const int g_res = (int)std::min<int64_t>((ctx->n_nodes + 7) / 8, (int64_t)ctx->sm_count * 8);
  if ((size_t)g_res * 2 * NR > ctx->partial_slots) return set_error(ctx, AXIA_ERR_TOO_LARGE, "partials area too small");
  const BsrMatM<float> M32{(int)ctx->n_nodes, ctx->d_qptr, ctx->d_qadj, ctx->d_bval32, (long long)ctx->nbq};
  const BsrMatM<double> M64{(int)ctx->n_nodes, ctx->d_qptr, ctx->d_qadj, ctx->d_bval64, (long long)ctx->nbq};
  BatchState hs;
  bool fp64_only = false;
  P.resume = 0;
  for (int seg = 0; seg < 100000; ++seg) {
    const int phase_unset = -1;
    AXIA_CUDA(ctx, cudaMemcpyAsync(&P.state->phase, &phase_unset, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    AXIA_CUDA(ctx, cudaMemsetAsync(ctx->d_bar, 0, sizeof(GridBarrier), ctx->stream));
    AXIA_TRY(launch_batch(ctx, kern, grid, P));
    AXIA_CUDA(ctx, cudaMemcpyAsync(&hs, P.state, sizeof(BatchState), cudaMemcpyDeviceToHost, ctx->stream));
    AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (hs.phase != 1) return AXIA_OK;  // finished, or stopped early (status / barrier limit)
    auto residual = [&](bool dwr, unsigned cases) -> int {
      if (dwr)
        k_batch_resid<true><<<g_res, 256, 0, ctx->stream>>>(M32, ctx->d_bval32lo, M64, ctx->d_mB, ctx->d_mX,
                                                             ctx->d_mXh, ctx->d_mXl, ctx->d_bdinv32, ctx->d_mR32,
                                                             ctx->d_partials, cases);
      else
        k_batch_resid<false><<<g_res, 256, 0, ctx->stream>>>(M32, ctx->d_bval32lo, M64, ctx->d_mB, ctx->d_mX,
                                                              ctx->d_mXh, ctx->d_mXl, ctx->d_bdinv32, ctx->d_mR32,
                                                              ctx->d_partials, cases);
      k_batch_resid_sum<<<2, NR * 32, 0, ctx->stream>>>(ctx->d_partials, g_res, ctx->d_totals);
      ctx->launches += 2;
      AXIA_CUDA(ctx, cudaGetLastError());
      return AXIA_OK;
    };
    k_batch_fold<<<ctx->sm_count * 8, 256, 0, ctx->stream>>>(n, ctx->d_mX, ctx->d_mX32, ctx->d_mXh, ctx->d_mXl,
                                                            fp64_only ? 0 : 1);
    ctx->launches++;
    AXIA_TRY(residual(!fp64_only, ~0u));
    if (!fp64_only) {
      double tot[NR];
      AXIA_CUDA(ctx, cudaMemcpyAsync(tot, ctx->d_totals, sizeof(tot), cudaMemcpyDeviceToHost, ctx->stream));
      AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      // the cases whose double-word residual meets tol or stalled: FP64 for them
      unsigned check = 0;
      for (int c = 0; c < NR; ++c) {
        if (!hs.active[c]) continue;
        const double rn = std::sqrt(tot[c]);
        if (rn <= P.tol * hs.bnorm[c] || !(rn <= 0.5 * hs.rmax[c])) check |= 1u << c;
      }
      if (check) {
        double t64[NR];
        CaseList list{};
        for (int c = 0; c < NR; ++c)
          if ((check >> c) & 1u) list.c[list.n++] = c;
        int kp = 1;
        while (kp < list.n) kp <<= 1;
        auto sub = [&](auto kern) {
          kern<<<g_res, 256, 0, ctx->stream>>>(M64, ctx->d_mB, ctx->d_mX, ctx->d_bdinv32, ctx->d_mR32,
                                               ctx->d_partials, list);
        };
        switch (kp) {
          case 1: sub(k_batch_resid64_cases<1>); break;
          case 2: sub(k_batch_resid64_cases<2>); break;
          case 4: sub(k_batch_resid64_cases<4>); break;
          case 8: sub(k_batch_resid64_cases<8>); break;
          case 16: sub(k_batch_resid64_cases<16>); break;
          default: sub(k_batch_resid64_cases<32>); break;
        }
        k_batch_resid_sum<<<2, NR * 32, 0, ctx->stream>>>(ctx->d_partials, g_res, ctx->d_totals);
        ctx->launches += 2;
        AXIA_CUDA(ctx, cudaGetLastError());
        AXIA_CUDA(ctx, cudaMemcpyAsync(t64, ctx->d_totals, sizeof(t64), cudaMemcpyDeviceToHost, ctx->stream));
        AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        // double-word and FP64 residuals apart by more than 10 %: the floor is reached
        for (int c = 0; c < NR; ++c) {
          if (!((check >> c) & 1u)) continue;
          const double a = std::sqrt(tot[c]), b = std::sqrt(t64[c]);
          if (!(std::fabs(a - b) <= 0.1 * b)) fp64_only = true;
        }
      }
    }
    P.resume = 1;
  }
  return set_error(ctx, AXIA_ERR_NOT_CONVERGED, "batched CG: too many segments");
}

int batch_solve(axia_ctx* ctx, int nrhs, const double* d_F, double* d_U, const axia_solve_opts* opts,
                axia_solve_info* info, double* rel_res) {
  if (!ctx->have_bsr64 || !ctx->have_bsr32)
    return set_error(ctx, AXIA_ERR_STATE, "batched solve needs the node-block forms (AXIA_ASM_BSR64 | AXIA_ASM_BSR32)");
  const int64_t nd = ctx->ndof;
  AXIA_TRY(ensure_batch_buffers(ctx));
  if (opts->preconditioner != AXIA_PRECOND_JACOBI && opts->preconditioner != AXIA_PRECOND_COARSE)
    return set_error(ctx, AXIA_ERR_INVALID_ARG, "batched load cases: unknown preconditioner");
  const bool coarse = opts->preconditioner == AXIA_PRECOND_COARSE;
  CoarseArgs cargs{};
  if (coarse) AXIA_TRY(coarse_prepare_batched(ctx, opts->coarse_nodes, &cargs));
  const long long max_iter = opts->max_iter > 0 ? opts->max_iter : std::max<long long>(4LL * ctx->n_free, 200);
  const double delta = opts->inner_rtol > 0 && opts->inner_rtol < 1 ? opts->inner_rtol : 0.01;
  const BatchTile tile = valid_tile(ctx->tuned_btc, ctx->tuned_btu) ? BatchTile{ctx->tuned_btc, ctx->tuned_btu}
                                                                     : kBatchDefault;
  const void* kern = coarse ? batch_kernel<true>(tile) : batch_kernel<false>(tile);
  int grid = 0;
  AXIA_TRY(batch_grid(ctx, kern, &grid));
  // with the FP32 low parts assembled the reliable updates run in double words
  // between segments of the kernel
  const bool split = ctx->have_bsr32lo;
  if (split) AXIA_TRY(ensure_segment_buffers(ctx));
  info->iters = 0;
  info->outer_iters = 0;
  double worst = 0.0;
  for (int c0 = 0; c0 < nrhs; c0 += NR) {
    const int nc = std::min(NR, nrhs - c0);
    AXIA_TRY(reset_dev_status(ctx));
    k_batch_rhs<<<ctx->sm_count * 8, 256, 0, ctx->stream>>>(nd, nc, ctx->d_ind_of, d_F + (int64_t)c0 * nd, ctx->d_kfu0,
                                                           ctx->d_mB);
    ctx->launches++;
    AXIA_CUDA(ctx, cudaMemsetAsync(ctx->d_bar, 0, sizeof(GridBarrier), ctx->stream));
    MultiArgs P = multi_args(ctx, opts->rtol, delta, max_iter, cargs);
    if (split) {
      P.state = static_cast<BatchState*>(ctx->d_mstate);
      P.split = 1;
      AXIA_TRY(timed_launch(ctx, info, [&]() -> int { return run_segmented(ctx, kern, grid, P); }));
    } else {
      AXIA_TRY(timed_launch(ctx, info, [&]() -> int { return launch_batch(ctx, kern, grid, P); }));
    }
    MultiOut o;
    AXIA_CUDA(ctx, cudaMemcpyAsync(&o, ctx->d_mout, sizeof(MultiOut), cudaMemcpyDeviceToHost, ctx->stream));
    AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    DevStatus hs;
    AXIA_TRY(read_dev_status(ctx, &hs));
    if (hs.timeout) return set_error(ctx, AXIA_ERR_TIMEOUT, "a grid barrier of the batched PCG ran past its limit");
    info->iters = std::max<int64_t>(info->iters, o.iters);
    info->outer_iters += o.updates;
    for (int c = 0; c < nc; ++c) {
      const double rr = o.bnorm[c] > 0 ? o.residual[c] / o.bnorm[c] : 0.0;
      if (rel_res) rel_res[c0 + c] = rr;
      worst = std::max(worst, rr);
    }
    if (o.status != AXIA_OK) {
      if (o.status == AXIA_ERR_ZERO_PIVOT) return set_error(ctx, o.status, "batched CG: zero pivot in a load case");
      return set_error(ctx, o.status, "batched CG did not converge in " + std::to_string(o.iters) + " iterations");
    }
    k_batch_out<<<ctx->sm_count * 8, 256, 0, ctx->stream>>>(nd, nc, ctx->d_ind_of, ctx->d_u0, ctx->d_mX,
                                                           d_U + (int64_t)c0 * nd);
    ctx->launches++;
    AXIA_CUDA(ctx, cudaGetLastError());
  }
  info->residual = worst;
  info->bnorm = 1.0;
  return AXIA_OK;
}
