// coarse.cu -- setup of the coarse space of the two-level preconditioner
// (the per-iteration phases are in coarse.cuh).
//
// No reference counterpart: the reference preconditions its CG with the
// diagonal only (solver/src/linalg.rs:199-259).
//
// Space (once per mesh and constraint set):
//   * bounding box -> a uniform grid of at most COARSE_MAX / 6 boxes of about
//     `nodes_target` nodes each; every non-empty box is a subdomain;
//   * the nodes sorted by subdomain (stable radix sort: ascending node order
//     inside each subdomain), cut into chunks of COARSE_CHUNK nodes;
//   * centre c_I, and per node (x_a - c_I) / h and its free-DOF mask (geo);
//   * per subdomain the Gram matrix G = Z_I^T Z_I over the free DOFs and
//     T = L^-T from its Cholesky factor, modes whose pivot vanishes dropped
//     (a subdomain with few free nodes has dependent rigid-body modes).
// Operator (after every assembly, from the FP64 node-block matrix):
//   * every node row a that is not interior to its subdomain: for each
//     subdomain J its blocks reach, Z_a^T sum_{b in row a, b in J} K_ab Z_b
//     (6 x 6, FP64); rows are split into items keyed (I(a), J), written in
//     row order;
//   * a stable radix sort by key, then every run summed in item order gives
//     S_IJ = Z_I^T K Z_J; A_IJ = T_I^T S_IJ T_J goes into a dense FP64 matrix;
//   * A scaled to unit diagonal, rounded to FP32 and inverted in place by a
//     symmetric blocked Gauss-Jordan elimination (64 x 64 tiles, one
//     cooperative launch, three bounded grid barriers per tile step, the next
//     pivot tile inverted during the current trailing update);
//   * M = T diag(s) A^-1 diag(s) T^T per subdomain pair, in FP32.
// Every sum has a fixed order: the same inputs give the same bits.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <cub/cub.cuh>

#include "coarse.cuh"

namespace {

constexpr int GJ_T = 64;          // Gauss-Jordan tile
constexpr int GJ_THREADS = 256;   // 16 x 16 threads, 4 x 4 outputs each
constexpr int ROW_SLOTS = 8;      // subdomains accumulated per pass over a node row
constexpr int GJ_GROUPS = 32;     // at most this many coarse blocks are inverted side by side

// One diagonal block of the coarse matrix: the unknowns [u0, u0 + n) of the
// subdomains s0 .. s0 + n / 6 - 1, padded to p (a multiple of GJ_T), stored
// as a dense p x p matrix at element offset off of a64 / a32 / minv.  One
// block holds every subdomain, unless the space is built for a multi-mesh
// solve: then each mesh has its own block (the meshes do not couple).
struct CoarseBlk {
  int u0, n, p, s0;
  long long off;
};

struct CoarseState {
  int nodes_target = 0;
  bool per_mesh = false;         // one block per mesh
  std::vector<CoarseBlk> blk;
  CoarseBlk* d_blk = nullptr;    // [n_blocks]
  int* d_sub_blk = nullptr;      // [n_sub] block of every subdomain
  long long blk_elems = 0;       // sum of p^2
  int max_p = 0;
  int64_t op_gen = -1;           // assembly the operator was built from
  CoarseArgs args{};
  double h = 0.0;
  int* sub_node = nullptr;
  int4* chunk = nullptr;
  int* chunk_ptr = nullptr;
  float4* geo = nullptr;
  int* sub_ptr = nullptr;        // [n_sub + 1]
  double* tmat = nullptr;        // [n_sub][6][6]
  float* minv = nullptr;         // [blk_elems] block by block, p x p each
  // operator scratch, kept for the rebuilds after every assembly
  std::vector<int> h_chunk_ptr;  // [n_sub + 1]
  std::vector<int> mesh_sub;     // [n_meshes + 1] subdomains of each mesh (one mesh: 0, n_sub)
  int* off = nullptr;            // [n_nodes + 1] first item of each node row
  unsigned* keys = nullptr;      // [n_items] subdomain pair I * n_sub + J
  double* vals = nullptr;        // [n_items][36]
  int* perm = nullptr;           // [n_items] items in (I, J) order (stable)
  unsigned* run_key = nullptr;   // [n_runs]
  int* run_off = nullptr;        // [n_runs]
  int* run_cnt = nullptr;        // [n_runs]
  int n_items = 0, n_runs = 0;
  bool items_fresh = false;      // vals already hold the current K's items
  double* a64 = nullptr;         // [blk_elems]
  float* a32 = nullptr;          // [blk_elems] inverted in place
  double* scale = nullptr;       // [ncp] per unknown
  float* piv = nullptr;          // [GJ_GROUPS][2][GJ_T][GJ_T]
  GridBarrier* gj_bar = nullptr; // [GJ_GROUPS]
  float* part = nullptr;         // [n_chunks][6]
  float* rc = nullptr;           // [ncp]
  int* cnt = nullptr;            // [n_sub]
  float* part_m = nullptr;       // [n_chunks][6][32] (batched solve)
  float* rc_m = nullptr;         // [ncp][32]
  float* yc_m = nullptr;         // [ncp][32]
  float* yc = nullptr;           // [ncp]
  void release(axia_ctx* ctx) {
    dev_release(ctx, sub_node);
    dev_release(ctx, chunk);
    dev_release(ctx, chunk_ptr);
    dev_release(ctx, geo);
    dev_release(ctx, sub_ptr);
    dev_release(ctx, tmat);
    dev_release(ctx, minv);
    dev_release(ctx, off);
    dev_release(ctx, keys);
    dev_release(ctx, vals);
    dev_release(ctx, perm);
    dev_release(ctx, run_key);
    dev_release(ctx, run_off);
    dev_release(ctx, run_cnt);
    dev_release(ctx, a64);
    dev_release(ctx, a32);
    dev_release(ctx, scale);
    dev_release(ctx, piv);
    dev_release(ctx, gj_bar);
    dev_release(ctx, part_m);
    dev_release(ctx, rc_m);
    dev_release(ctx, yc_m);
    dev_release(ctx, part);
    dev_release(ctx, rc);
    dev_release(ctx, cnt);
    dev_release(ctx, yc);
    dev_release(ctx, d_blk);
    dev_release(ctx, d_sub_blk);
  }
};

// ---------------------------------------------------------------------------
// Space
// ---------------------------------------------------------------------------
__global__ void k_bbox(int64_t a0, int64_t a1, const double* __restrict__ xyz, double* out) {
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t a = a0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < a1; a += (int64_t)gridDim.x * blockDim.x)
    for (int d = 0; d < 3; ++d) {
      const double v = xyz[3 * a + d];
      lo[d] = fmin(lo[d], v);
      hi[d] = fmax(hi[d], v);
    }
  __shared__ double s[6][32];
  for (int d = 0; d < 3; ++d) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[d] = fmin(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
      hi[d] = fmax(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
    }
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0)
    for (int d = 0; d < 3; ++d) {
      s[d][w] = lo[d];
      s[3 + d][w] = hi[d];
    }
  __syncthreads();
  if (threadIdx.x < 6) {
    double v = s[threadIdx.x][0];
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k)
      v = threadIdx.x < 3 ? fmin(v, s[threadIdx.x][k]) : fmax(v, s[threadIdx.x][k]);
    out[6 * blockIdx.x + threadIdx.x] = v;
  }
}

struct Grid3 {
  double x0, y0, z0, h;
  int nx, ny, nz;
};

__device__ __forceinline__ int cell_of(const Grid3& g, double x, double y, double z) {
  const int ix = min(max((int)floor((x - g.x0) / g.h), 0), g.nx - 1);
  const int iy = min(max((int)floor((y - g.y0) / g.h), 0), g.ny - 1);
  const int iz = min(max((int)floor((z - g.z0) / g.h), 0), g.nz - 1);
  return ix + g.nx * (iy + g.ny * iz);
}

// cells of the nodes [a0, a1) (one mesh) in the grid g, numbered from base
__global__ void k_cell_count(int64_t a0, int64_t a1, const double* __restrict__ xyz, Grid3 g, int base, int* cell,
                             int* count) {
  for (int64_t a = a0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < a1; a += (int64_t)gridDim.x * blockDim.x) {
    const int c = base + cell_of(g, xyz[3 * a], xyz[3 * a + 1], xyz[3 * a + 2]);
    cell[a] = c;
    atomicAdd(count + c, 1);
  }
}

__global__ void k_sub_of_node(int64_t n, const int* cell, const int* cell_sub, int* sub, int* iota) {
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < n; a += (int64_t)gridDim.x * blockDim.x) {
    sub[a] = cell_sub[cell[a]];
    iota[a] = (int)a;
  }
}

// warp per subdomain: centre = mean of its node coordinates (fixed lane order)
__global__ void k_sub_centre(int n_sub, const int* sub_ptr, const int* sub_node, const double* __restrict__ xyz,
                             double* centre) {
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; I < n_sub; I += nw) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    const int b = sub_ptr[I], e = sub_ptr[I + 1];
    for (int k = b + lane; k < e; k += 32) {
      const int a = sub_node[k];
      s0 += xyz[3 * a];
      s1 += xyz[3 * a + 1];
      s2 += xyz[3 * a + 2];
    }
    s0 = warp_sum(s0);
    s1 = warp_sum(s1);
    s2 = warp_sum(s2);
    if (lane == 0) {
      const double inv = 1.0 / (double)(e - b);
      centre[3 * I] = s0 * inv;
      centre[3 * I + 1] = s1 * inv;
      centre[3 * I + 2] = s2 * inv;
    }
  }
}

__global__ void k_geo(int64_t n, const double* __restrict__ xyz, const int* sub, const double* centre,
                      const double* sub_inv_h, const int32_t* ind_of, float4* geo) {
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < n; a += (int64_t)gridDim.x * blockDim.x) {
    const int I = sub[a];
    const double inv_h = sub_inv_h[I];
    unsigned m = 0;
    for (int d = 0; d < 3; ++d)
      if (ind_of[3 * a + d] >= 0) m |= 1u << d;
    geo[a] = make_float4((float)((xyz[3 * a] - centre[3 * I]) * inv_h),
                         (float)((xyz[3 * a + 1] - centre[3 * I + 1]) * inv_h),
                         (float)((xyz[3 * a + 2] - centre[3 * I + 2]) * inv_h), __uint_as_float(((unsigned)I << 3) | m));
  }
}

// rows of Z_a (masked): row d of the 3 x 6 block, in double
__device__ __forceinline__ void z_row(float4 g, int d, double r[6]) {
  const unsigned m = geo_bits(g);
  const double X = g.x, Y = g.y, Z = g.z;
  for (int k = 0; k < 6; ++k) r[k] = 0.0;
  if (!(m & (1u << d))) return;
  r[d] = 1.0;
  if (d == 0) {
    r[4] = Z;
    r[5] = -Y;
  } else if (d == 1) {
    r[3] = -Z;
    r[5] = X;
  } else {
    r[3] = Y;
    r[4] = -X;
  }
}

// warp per subdomain: G = Z_I^T Z_I, then T = L^-T on the kept modes
__global__ void k_sub_gram(int n_sub, const int* sub_ptr, const int* sub_node, const float4* geo, double* tmat) {
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; I < n_sub; I += nw) {
    double G[21];
    for (int k = 0; k < 21; ++k) G[k] = 0.0;
    for (int k = sub_ptr[I] + lane; k < sub_ptr[I + 1]; k += 32) {
      const float4 g = geo[sub_node[k]];
      for (int d = 0; d < 3; ++d) {
        double r[6];
        z_row(g, d, r);
        int q = 0;
        for (int i = 0; i < 6; ++i)
          for (int j = 0; j <= i; ++j, ++q) G[q] = fma(r[i], r[j], G[q]);
      }
    }
    for (int k = 0; k < 21; ++k) G[k] = warp_sum(G[k]);
    if (lane == 0) {
      double A[6][6], L[6][6] = {}, Li[6][6] = {};
      int q = 0;
      for (int i = 0; i < 6; ++i)
        for (int j = 0; j <= i; ++j, ++q) A[i][j] = A[j][i] = G[q];
      double gmax = 0.0;
      for (int i = 0; i < 6; ++i) gmax = fmax(gmax, A[i][i]);
      bool keep[6];
      for (int j = 0; j < 6; ++j) {
        double d = A[j][j];
        for (int k = 0; k < j; ++k) d -= L[j][k] * L[j][k];
        keep[j] = gmax > 0.0 && d > 1e-9 * gmax;
        if (!keep[j]) continue;
        L[j][j] = sqrt(d);
        for (int i = j + 1; i < 6; ++i) {
          double s = A[i][j];
          for (int k = 0; k < j; ++k) s -= L[i][k] * L[j][k];
          L[i][j] = s / L[j][j];
        }
      }
      for (int c = 0; c < 6; ++c) {
        if (!keep[c]) continue;
        Li[c][c] = 1.0 / L[c][c];
        for (int i = c + 1; i < 6; ++i) {
          if (!keep[i]) continue;
          double s = 0.0;
          for (int k = c; k < i; ++k)
            if (keep[k]) s += L[i][k] * Li[k][c];
          Li[i][c] = -s / L[i][i];
        }
      }
      for (int k = 0; k < 6; ++k)
        for (int i = 0; i < 6; ++i) tmat[36 * I + 6 * k + i] = Li[i][k];  // T = Li^T
    }
  }
}

// ---------------------------------------------------------------------------
// Operator
// ---------------------------------------------------------------------------

// A node row whose blocks all lie in its own subdomain, with every DOF of
// the row's nodes free, contributes Z_a^T (K Z_I)_a = 0: the element
// stiffnesses annihilate rigid-body motions (up to the rounding of geo), so
// the row is left out.  Same test in the count and in the fill.
__device__ __forceinline__ bool row_is_interior(int beg, int end, const int* __restrict__ adj, const float4* geo,
                                                unsigned ma, int lane) {
  const unsigned want = (ma & ~7u) | 7u;
  if (ma != want) return false;
  bool ok = true;
  for (int s = beg + lane; s < end; s += 32) ok = ok && geo_bits(__ldg(geo + __ldg(adj + s))) == want;
  return __all_sync(0xffffffffu, ok);
}

// The distinct subdomains of a node row's blocks, in order of first
// appearance; lane k holds the k-th.  Returns their count (> 32: overflow).
__device__ __forceinline__ int row_subdomains(int beg, int end, const int* __restrict__ adj, const float4* geo,
                                              int lane, int* mine) {
  int n = 0;
  *mine = -1;
  for (int s0 = beg; s0 < end; s0 += 32) {
    const int s = s0 + lane;
    const int J = s < end ? (int)(geo_bits(__ldg(geo + __ldg(adj + s))) >> 3) : -1;
    unsigned pending = __ballot_sync(0xffffffffu, J >= 0);
    while (pending) {
      const int l = __ffs(pending) - 1;
      const int Jl = __shfl_sync(0xffffffffu, J, l);
      const bool have = __ballot_sync(0xffffffffu, lane < n && *mine == Jl) != 0;
      if (!have) {
        if (lane == n) *mine = Jl;
        ++n;
      }
      pending &= ~__ballot_sync(0xffffffffu, J == Jl);
    }
  }
  return n;
}

__global__ void k_row_count(int n_nodes, const int* __restrict__ ptr, const int* __restrict__ adj, const float4* geo,
                            int* cnt, DevStatus* st) {
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; a < n_nodes; a += nw) {
    const int beg = __ldg(ptr + a), end = __ldg(ptr + a + 1);
    int n = 0;
    if (!row_is_interior(beg, end, adj, geo, geo_bits(__ldg(geo + a)), lane)) {
      int mine;
      n = row_subdomains(beg, end, adj, geo, lane, &mine);
    }
    if (n > ROW_SLOTS * 4 && lane == 0) record_error(st, a, AXIA_ERR_INVALID_ARG);
    if (lane == 0) cnt[a] = min(n, ROW_SLOTS * 4);
  }
}

constexpr int ROW_WARPS = 8;
constexpr int WS = 19;  // padded stride of a lane's 18 W entries in shared memory

// Items of row a: for each subdomain J its blocks reach,
//   W = sum_{b in J} M_a K_ab M_b Z_b   (3 x 6, M = free-DOF masks; lane e < 18
// holds entry e, summed over the row's blocks in order), then C = Z_a^T W.
// V = float reads the FP32 matrix and computes on the FP32 pipe (the operator
// is inverted in FP32 anyway; FP64 bounded this kernel on GB300), double the
// FP64 matrix (when no FP32 node-block form is assembled).
template <typename V>
__global__ void __launch_bounds__(32 * ROW_WARPS) k_row_items(int n_nodes, int n_sub, BsrMat<V> K,
                                                               const float4* geo, const int* __restrict__ off,
                                                               unsigned* keys, double* vals) {
  __shared__ V s_w[ROW_WARPS][32 * WS];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  V* sw = s_w[wid];
  const int nw = (gridDim.x * blockDim.x) >> 5;
  const long long nb = K.nb;
  for (int a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; a < n_nodes; a += nw) {
    const int o = __ldg(off + a), n = __ldg(off + a + 1) - o;
    if (n == 0) continue;  // interior row (warp-uniform)
    const int beg = __ldg(K.adj_ptr + a), end = __ldg(K.adj_ptr + a + 1);
    int mine;
    row_subdomains(beg, end, K.adj, geo, lane, &mine);
    const float4 ga = __ldg(geo + a);
    const unsigned ma = geo_bits(ga);
    const int I = (int)(ma >> 3);
    for (int g0 = 0; g0 < n; g0 += ROW_SLOTS) {
      V acc[ROW_SLOTS];
#pragma unroll
      for (int k = 0; k < ROW_SLOTS; ++k) acc[k] = V(0);
      for (int s0 = beg; s0 < end; s0 += 32) {
        const int s = s0 + lane;
        int J = -1;
        if (s < end) {
          const int b = __ldg(K.adj + s);
          const float4 gb = __ldg(geo + b);
          const unsigned mb = geo_bits(gb);
          J = (int)(mb >> 3);
          V Kc[3][3];
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
              const V v = __ldg(K.val + (3 * i + j) * nb + s);
              Kc[i][j] = ((ma >> i) & (mb >> j) & 1u) ? v : V(0);
            }
          const V Xb = gb.x, Yb = gb.y, Zb = gb.z;
          V* w = sw + lane * WS;
#pragma unroll
          for (int i = 0; i < 3; ++i) {  // row i of Kc Z_b
            w[6 * i + 0] = Kc[i][0];
            w[6 * i + 1] = Kc[i][1];
            w[6 * i + 2] = Kc[i][2];
            w[6 * i + 3] = fma(Yb, Kc[i][2], -Zb * Kc[i][1]);
            w[6 * i + 4] = fma(Zb, Kc[i][0], -Xb * Kc[i][2]);
            w[6 * i + 5] = fma(Xb, Kc[i][1], -Yb * Kc[i][0]);
          }
        }
        __syncwarp();
#pragma unroll
        for (int k = 0; k < ROW_SLOTS; ++k) {
          if (g0 + k >= n) break;
          const int Jk = __shfl_sync(0xffffffffu, mine, g0 + k);
          for (unsigned m = __ballot_sync(0xffffffffu, J == Jk); m; m &= m - 1) {
            const int l = __ffs(m) - 1;
            if (lane < 18) acc[k] += sw[l * WS + lane];
          }
        }
        __syncwarp();
      }
      const V Xa = ga.x, Ya = ga.y, Za = ga.z;
#pragma unroll
      for (int k = 0; k < ROW_SLOTS; ++k) {
        if (g0 + k >= n) break;
        const int Jk = __shfl_sync(0xffffffffu, mine, g0 + k);
        const int item = o + g0 + k;
        if (lane == 0) keys[item] = (unsigned)I * (unsigned)n_sub + (unsigned)Jk;
        // C[i][j] = (Z_a^T W)[i][j]; W[r][j] sits on lane 6 r + j
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int e = lane + 32 * h;
          const int j = (e < 36 ? e : 0) % 6, i = (e < 36 ? e : 0) / 6;
          const V w0 = __shfl_sync(0xffffffffu, acc[k], j);
          const V w1 = __shfl_sync(0xffffffffu, acc[k], 6 + j);
          const V w2 = __shfl_sync(0xffffffffu, acc[k], 12 + j);
          V c = i == 0 ? w0 : i == 1 ? w1 : i == 2 ? w2
              : i == 3 ? fma(Ya, w2, -Za * w1) : i == 4 ? fma(Za, w0, -Xa * w2) : fma(Xa, w1, -Ya * w0);
          if (e < 36) vals[(size_t)item * 36 + e] = (double)c;
        }
      }
    }
  }
}

// warp per run of equal (I, J): S = sum of its items in sorted order, then
// A_IJ = T_I^T S T_J into the dense matrix (row stride ld)
__global__ void k_run_sum(int n_runs, int n_sub, const unsigned* run_key, const int* run_off, const int* run_cnt,
                          const int* perm, const double* __restrict__ vals, const double* __restrict__ tmat,
                          double* A, const CoarseBlk* blk, const int* sub_blk) {
  __shared__ double s_S[8][36], s_U[8][36];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n_runs; r += nw) {
    const int I = (int)(run_key[r] / (unsigned)n_sub), J = (int)(run_key[r] % (unsigned)n_sub);
    const CoarseBlk B = blk[sub_blk[I]];
    if (sub_blk[J] != sub_blk[I]) continue;  // never: the blocks (meshes) do not couple
    const int b = run_off[r], e = b + run_cnt[r];
    double s0 = 0.0, s1 = 0.0;
#pragma unroll 4
    for (int k = b; k < e; ++k) {
      const double* v = vals + (size_t)perm[k] * 36;
      s0 += v[lane];
      if (lane < 4) s1 += v[32 + lane];
    }
    s_S[w][lane] = s0;
    if (lane < 4) s_S[w][32 + lane] = s1;
    __syncwarp();
    const double* TI = tmat + 36 * I;
    const double* TJ = tmat + 36 * J;
    // U = S T_J
    for (int q = lane; q < 36; q += 32) {
      const int k = q / 6, j = q % 6;
      double u = 0.0;
      for (int l = 0; l < 6; ++l) u = fma(s_S[w][6 * k + l], TJ[6 * l + j], u);
      s_U[w][q] = u;
    }
    __syncwarp();
    for (int q = lane; q < 36; q += 32) {
      const int i = q / 6, j = q % 6;
      double v = 0.0;
      for (int k = 0; k < 6; ++k) v = fma(TI[6 * k + i], s_U[w][6 * k + j], v);
      A[B.off + (size_t)(6 * I + i - B.u0) * B.p + 6 * J + j - B.u0] = v;
    }
    __syncwarp();
  }
}

// block blockIdx.y: B = diag(s) A diag(s) in FP32; unknowns without a scale
// (dropped modes, padding) become identity rows and columns
__global__ void k_scale_to_f32(const CoarseBlk* blk, const double* A, const double* scale, float* B) {
  const CoarseBlk K = blk[blockIdx.y];
  const int64_t n2 = (int64_t)K.p * K.p;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n2; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t / K.p), j = (int)(t % K.p);
    const double si = i < K.n ? scale[K.u0 + i] : 0.0, sj = j < K.n ? scale[K.u0 + j] : 0.0;
    B[K.off + t] = (si == 0.0 || sj == 0.0) ? (i == j ? 1.0f : 0.0f) : (float)(A[K.off + t] * si * sj);
  }
}

// ---------------------------------------------------------------------------
// Blocked Gauss-Jordan inverse of an SPD matrix (FP32, in place, no pivoting).
// Step k with P = A_kk^-1 and the new row panel R_j = P A_kj (j != k):
//   A_ij <- A_ij - A_ik R_j  (i, j != k),  A_kj <- R_j,  A_ik <- -R_i^T,  A_kk <- P.
// With S_i = -1 for the block indices eliminated so far and +1 for the rest,
// every intermediate satisfies A_ij = S_i S_j A_ji^T (the final inverse,
// S = -1 throughout, is symmetric).  So the trailing update runs over the
// tiles with j <= i and mirrors them with that sign, and the new column panel
// is A_ik = -S_i R_i^T.
// ---------------------------------------------------------------------------
constexpr int GJ_LD = GJ_T + 4;   // shared-memory row stride (16-byte aligned rows)

struct GjArgs {
  float* A;
  int n;             // multiple of GJ_T
  float* piv;        // [2][GJ_T][GJ_T] P of step k in buffer k & 1
  GridBarrier* bar;
  DevStatus* st;
  unsigned long long limit_ns;
  int rank, nb;      // this block's rank in its group of nb blocks (at least 2)
};

// operand tiles: sa[q][r] = X[r][q] (transposed), sb[q][c] = Y[q][c]
__device__ __forceinline__ void gj_load_t(float (*sa)[GJ_LD], const float* g, int ld) {
  for (int t = threadIdx.x; t < GJ_T * GJ_T; t += blockDim.x) sa[t % GJ_T][t / GJ_T] = g[(size_t)(t / GJ_T) * ld + t % GJ_T];
}
__device__ __forceinline__ void gj_load(float (*sb)[GJ_LD], const float* g, int ld) {
  for (int t = threadIdx.x; t < GJ_T * GJ_T / 4; t += blockDim.x) {
    const int r = t / (GJ_T / 4), c = 4 * (t % (GJ_T / 4));
    *reinterpret_cast<float4*>(&sb[r][c]) = *reinterpret_cast<const float4*>(g + (size_t)r * ld + c);
  }
}

// out[4][4] = rows 4ty.. / cols 4tx.. of X Y
__device__ __forceinline__ void gj_mul(float (*sa)[GJ_LD], float (*sb)[GJ_LD], float out[4][4]) {
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) out[r][c] = 0.f;
#pragma unroll 8
  for (int q = 0; q < GJ_T; ++q) {
    const float4 x = *reinterpret_cast<const float4*>(&sa[q][4 * ty]);
    const float4 y = *reinterpret_cast<const float4*>(&sb[q][4 * tx]);
    const float xr[4] = {x.x, x.y, x.z, x.w}, yc[4] = {y.x, y.y, y.z, y.w};
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) out[r][c] = fmaf(xr[r], yc[c], out[r][c]);
  }
}

// thread (ty, tx)'s 4 x 4 part of a tile into registers
__device__ __forceinline__ void gj_load_regs(float (&a)[4][4], const float* g, int ld) {
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const float4 v = *reinterpret_cast<const float4*>(g + (size_t)(4 * ty + r) * ld + 4 * tx);
    a[r][0] = v.x;
    a[r][1] = v.y;
    a[r][2] = v.z;
    a[r][3] = v.w;
  }
}

// a dense 64 x 64 buffer into a tile of the matrix
__device__ __forceinline__ void gj_store_global(const float* src, float* g, int ld) {
  for (int t = threadIdx.x; t < GJ_T * GJ_T / 4; t += blockDim.x) {
    const int r = t / (GJ_T / 4), c = 4 * (t % (GJ_T / 4));
    *reinterpret_cast<float4*>(g + (size_t)r * ld + c) = *reinterpret_cast<const float4*>(src + (size_t)r * GJ_T + c);
  }
}

// column panel of step k: tile (i, k) = -S_i tile (k, i)^T (i != k; S_i = -1 for i < k)
__device__ __forceinline__ void gj_column_panel(const GjArgs& P, int k, int first, int stride) {
  const int nt = P.n / GJ_T, ld = P.n;
  for (int i = first; i < nt; i += stride) {
    if (i == k) continue;
    const float sg = i < k ? 1.f : -1.f;
    const float* src = P.A + (size_t)k * GJ_T * ld + (size_t)i * GJ_T;
    float* dst = P.A + (size_t)i * GJ_T * ld + (size_t)k * GJ_T;
    for (int t = threadIdx.x; t < GJ_T * GJ_T; t += blockDim.x) {
      const int r = t / GJ_T, c = t % GJ_T;  // coalesced reads of src row r
      dst[(size_t)c * ld + r] = sg * src[(size_t)r * ld + c];
    }
  }
}

// Gauss-Jordan inverse of one 64 x 64 SPD tile, the register form: the
// block's threads place their 4 x 4 parts in T (row stride GJ_LD); the 128
// threads of warps 0..3 then take half a column each (column j = tid % 64,
// rows 32 h .. 32 h + 31, h = tid / 64) into registers and run the 64 pivots
// fully unrolled.  Pivot p needs column p, A_ip = S_i A_pi with S_i = -1 for
// the pivots already taken (the sign structure of the symmetric elimination),
// and row p sits in half p / 32: its 64 threads publish S_j A_pj to cpiv
// (double-buffered) and a 128-thread named barrier per pivot.  Measured per
// 64 x 64 tile at 3072 unknowns: 26 us, against 47 us for all 256 threads on
// 4 x 4 parts with a block barrier per pivot and 33 us for the tile kept in
// shared memory with a rolled pivot loop; the inversion runs beside the
// trailing update of the step (34 us), so it is no longer the step's critical
// path.  The inverse is written to the 64 x 64 buffer out (row-major).
__device__ __forceinline__ void gj_invert_tile(const float (&a)[4][4], float* T, float* cpiv, float* out,
                                               DevStatus* st, int base) {
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
#pragma unroll
  for (int r = 0; r < 4; ++r)
    *reinterpret_cast<float4*>(T + (4 * ty + r) * GJ_LD + 4 * tx) = make_float4(a[r][0], a[r][1], a[r][2], a[r][3]);
  __syncthreads();
  if (threadIdx.x < 2 * GJ_T) {
    constexpr int HR = GJ_T / 2;  // rows per half
    const int j = threadIdx.x % GJ_T, h = threadIdx.x / GJ_T;
    float col[HR];
#pragma unroll
    for (int i = 0; i < HR; ++i) col[i] = T[(HR * h + i) * GJ_LD + j];
#pragma unroll
    for (int p = 0; p < GJ_T; ++p) {
      float* cp = cpiv + (p & 1) * GJ_T;
      const bool mine = (p / HR) == h;  // warp-uniform: row p is in this half
      if (mine) cp[j] = j < p ? -col[p % HR] : col[p % HR];
      asm volatile("bar.sync 1, 128;" ::: "memory");
      const float piv = cp[p];
      if (threadIdx.x == 0 && (!(piv > 0.f) || !isfinite(piv))) record_error(st, base + p, AXIA_ERR_ZERO_PIVOT);
      const float d = __frcp_rn(piv);
      const float rp = (j < p ? -cp[j] : cp[j]) * d;  // A_pj / A_pp
      const float* ch = cp + HR * h;
      if (j == p) {  // the pivot column: -A_ip / A_pp, and 1 / A_pp on the pivot
#pragma unroll
        for (int i4 = 0; i4 < HR; i4 += 4) {
          const float4 c4 = *reinterpret_cast<const float4*>(ch + i4);
          col[i4] = -c4.x * d;
          col[i4 + 1] = -c4.y * d;
          col[i4 + 2] = -c4.z * d;
          col[i4 + 3] = -c4.w * d;
        }
        if (mine) col[p % HR] = d;
      } else {
#pragma unroll
        for (int i4 = 0; i4 < HR; i4 += 4) {
          const float4 c4 = *reinterpret_cast<const float4*>(ch + i4);
          col[i4] = fmaf(-c4.x, rp, col[i4]);
          col[i4 + 1] = fmaf(-c4.y, rp, col[i4 + 1]);
          col[i4 + 2] = fmaf(-c4.z, rp, col[i4 + 2]);
          col[i4 + 3] = fmaf(-c4.w, rp, col[i4 + 3]);
        }
        if (mine) col[p % HR] = rp;
      }
    }
#pragma unroll
    for (int i = 0; i < HR; ++i) out[(HR * h + i) * GJ_T + j] = col[i];
  }
  __syncthreads();
}

__device__ __forceinline__ void gj_store_regs(const float (&a)[4][4], float* g, int ld) {
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
#pragma unroll
  for (int r = 0; r < 4; ++r)
    *reinterpret_cast<float4*>(g + (size_t)(4 * ty + r) * ld + 4 * tx) = make_float4(a[r][0], a[r][1], a[r][2], a[r][3]);
}

// Step k uses P_k = piv[k & 1].  The next pivot tile (k+1, k+1) is a trailing
// tile of step k: block 0 updates it alone and inverts it at once (lookahead)
// while the other blocks update the remaining tiles, so no step waits for a
// serial pivot inversion except the first.
// Inverts the n x n block at P.A in place; false when a barrier gave up.
__device__ __forceinline__ bool gj_invert_block(GjArgs P) {
  __shared__ __align__(16) float sa[GJ_T][GJ_LD];
  __shared__ __align__(16) float sb[GJ_T][GJ_LD];
  const int nt = P.n / GJ_T, ld = P.n;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  auto tile = [&](int i, int j) { return P.A + (size_t)i * GJ_T * ld + (size_t)j * GJ_T; };
  auto piv = [&](int k) { return P.piv + (size_t)(k & 1) * GJ_T * GJ_T; };
  for (int k = 0; k < nt; ++k) {
    // 1. block 0 stores P_(k-1) into its tile (and inverts tile (0, 0) at
    //    k = 0); the other blocks write step k-1's column panel
    if (P.rank == 0) {
      if (k > 0) gj_store_global(piv(k - 1), tile(k - 1, k - 1), ld);
      if (k == 0) {
        float a[4][4];
        gj_load_regs(a, tile(0, 0), ld);
        gj_invert_tile(a, &sa[0][0], &sb[0][0], piv(0), P.st, 0);
      }
    } else if (k > 0) {
      gj_column_panel(P, k - 1, P.rank - 1, P.nb - 1);
    }
    if (!group_sync(P.bar, P.st, P.limit_ns, P.nb)) return false;
    // 2. row panel: A_kj <- P_k A_kj
    for (int j = P.rank; j < nt; j += P.nb) {
      if (j == k) continue;
      __syncthreads();
      gj_load_t(sa, piv(k), GJ_T);
      gj_load(sb, tile(k, j), ld);
      __syncthreads();
      float o[4][4];
      gj_mul(sa, sb, o);
      gj_store_regs(o, tile(k, j), ld);
    }
    if (!group_sync(P.bar, P.st, P.limit_ns, P.nb)) return false;
    // 3. trailing tiles j <= i (i, j != k): A_ij -= A_ik R_j, mirrored into
    //    A_ji; block 0 takes tile (k+1, k+1) alone and inverts it
    const int m = nt - 1, ntiles = m * (m + 1) / 2;
    const bool ahead = k + 1 < nt && P.nb > 1;
    const int tdiag = ahead ? k * (k + 1) / 2 + k : -1;  // (k+1, k+1) in the compressed numbering
    if (ahead && P.rank == 0) {
      __syncthreads();
      gj_load_t(sa, tile(k + 1, k), ld);
      gj_load(sb, tile(k, k + 1), ld);
      __syncthreads();
      float o[4][4], a[4][4];
      gj_mul(sa, sb, o);
      const float* g = tile(k + 1, k + 1);
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const float4 c = *reinterpret_cast<const float4*>(g + (size_t)(4 * ty + r) * ld + 4 * tx);
        a[r][0] = c.x - o[r][0];
        a[r][1] = c.y - o[r][1];
        a[r][2] = c.z - o[r][2];
        a[r][3] = c.w - o[r][3];
      }
      __syncthreads();  // sa / sb are reused as the tile and pivot-column buffers
      gj_invert_tile(a, &sa[0][0], &sb[0][0], piv(k + 1), P.st, (k + 1) * GJ_T);
    }
    const int first = ahead ? P.rank - 1 : P.rank;
    const int stride = ahead ? P.nb - 1 : P.nb;
    for (int t = first; first >= 0 && t < ntiles; t += stride) {
      if (t == tdiag) continue;
      int i = (int)((sqrtf(8.f * t + 1.f) - 1.f) * 0.5f);
      while (i * (i + 1) / 2 > t) --i;
      while ((i + 1) * (i + 2) / 2 <= t) ++i;
      int j = t - i * (i + 1) / 2;
      if (i >= k) ++i;
      if (j >= k) ++j;
      __syncthreads();
      gj_load_t(sa, tile(i, k), ld);
      gj_load(sb, tile(k, j), ld);
      __syncthreads();
      float o[4][4];
      gj_mul(sa, sb, o);
      float* g = tile(i, j);
      float v[4][4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const float4 c = *reinterpret_cast<const float4*>(g + (size_t)(4 * ty + r) * ld + 4 * tx);
        v[r][0] = c.x - o[r][0];
        v[r][1] = c.y - o[r][1];
        v[r][2] = c.z - o[r][2];
        v[r][3] = c.w - o[r][3];
        *reinterpret_cast<float4*>(g + (size_t)(4 * ty + r) * ld + 4 * tx) = make_float4(v[r][0], v[r][1], v[r][2], v[r][3]);
      }
      if (i != j) {  // A_ji = S_i S_j A_ij^T
        const float sg = (i < k) == (j < k) ? 1.f : -1.f;
        float* h = tile(j, i);
#pragma unroll
        for (int c = 0; c < 4; ++c)
          *reinterpret_cast<float4*>(h + (size_t)(4 * tx + c) * ld + 4 * ty) =
              make_float4(sg * v[0][c], sg * v[1][c], sg * v[2][c], sg * v[3][c]);
      }
    }
    if (!group_sync(P.bar, P.st, P.limit_ns, P.nb)) return false;
  }
  // the last step's P and column panel
  const int k = nt - 1;
  if (P.rank == 0) {
    gj_store_global(piv(k), tile(k, k), ld);
  } else {
    gj_column_panel(P, k, P.rank - 1, P.nb - 1);
  }
  return true;
}

// The diagonal blocks of the coarse matrix in one cooperative launch: the
// blocks are split into ngroups groups (block b to group b mod ngroups, the
// launch's blocks likewise by blockIdx mod ngroups); each group inverts its
// blocks one after another with its own barrier and pivot buffers (reused,
// hence the barrier between blocks).  Groups never wait on one another.
__global__ void __launch_bounds__(GJ_THREADS, 2) k_gj_inverse(GjArgs P, const CoarseBlk* blk, int nblk, int ngroups) {
  const int g = (int)(blockIdx.x % (unsigned)ngroups);
  GjArgs Q = P;
  Q.rank = (int)(blockIdx.x / (unsigned)ngroups);
  Q.nb = ((int)gridDim.x - g + ngroups - 1) / ngroups;
  Q.bar = P.bar + g;
  Q.piv = P.piv + (size_t)g * 2 * GJ_T * GJ_T;
  for (int b = g; b < nblk; b += ngroups) {
    if (b != g && !group_sync(Q.bar, Q.st, Q.limit_ns, Q.nb)) return;
    Q.A = P.A + blk[b].off;
    Q.n = blk[b].p;
    if (!gj_invert_block(Q)) return;
  }
}

// M_IJ = T_I diag(s_I) B_IJ diag(s_J) T_J^T in the raw mode basis (thread per pair)
__global__ void k_minv(const CoarseBlk* blk, const float* __restrict__ B, const double* __restrict__ scale,
                       const double* __restrict__ tmat, float* M) {
  const CoarseBlk K = blk[blockIdx.y];  // pairs of the subdomains of block blockIdx.y
  const int ns = K.n / 6, ncp = K.p;
  const int64_t npair = (int64_t)ns * ns;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < npair; t += (int64_t)gridDim.x * blockDim.x) {
    const int I = K.s0 + (int)(t / ns), J = K.s0 + (int)(t % ns);
    const double* TI = tmat + 36 * I;
    const double* TJ = tmat + 36 * J;
    double Bs[6][6];
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j)
        Bs[i][j] = (double)B[K.off + (size_t)(6 * I + i - K.u0) * ncp + 6 * J + j - K.u0] * scale[6 * I + i] *
                   scale[6 * J + j];
    // U[i][l] = sum_j Bs[i][j] T_J[l][j]
    double U[6][6];
    for (int i = 0; i < 6; ++i)
      for (int l = 0; l < 6; ++l) {
        double u = 0.0;
        for (int j = 0; j < 6; ++j) u = fma(Bs[i][j], TJ[6 * l + j], u);
        U[i][l] = u;
      }
    for (int k = 0; k < 6; ++k)
      for (int l = 0; l < 6; ++l) {
        double v = 0.0;
        for (int i = 0; i < 6; ++i) v = fma(TI[6 * k + i], U[i][l], v);
        M[K.off + (size_t)(6 * I + k - K.u0) * ncp + 6 * J + l - K.u0] = (float)v;
      }
  }
}

int read_status(axia_ctx* ctx, const char* what) {
  DevStatus hs;
  AXIA_TRY(read_dev_status(ctx, &hs));
  if (hs.first_error != ~0ull) {
    ctx->last_bad = (int64_t)(hs.first_error >> 8);
    return set_error(ctx, (int)(hs.first_error & 0xff), std::string("coarse space: ") + what);
  }
  if (hs.timeout) return set_error(ctx, AXIA_ERR_TIMEOUT, std::string("coarse space: barrier timeout in ") + what);
  return AXIA_OK;
}

template <typename T>
int copy_to_host(axia_ctx* ctx, T* h, const T* d, size_t n) {
  AXIA_CUDA(ctx, cudaMemcpyAsync(h, d, n * sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
  AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return AXIA_OK;
}

template <typename T>
int copy_to_device(axia_ctx* ctx, T* d, const T* h, size_t n) {
  AXIA_CUDA(ctx, cudaMemcpyAsync(d, h, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
  AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return AXIA_OK;
}

int grid_for(const axia_ctx* ctx, int64_t n, int threads) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads, (int64_t)ctx->sm_count * 16));
}

// subdomains, chunks, geo and T for the current mesh and constraints
int build_space(axia_ctx* ctx, CoarseState* S) {
  const int64_t n = ctx->n_nodes;
  if (n >= (1LL << 28)) return set_error(ctx, AXIA_ERR_TOO_LARGE, "coarse space: too many nodes");
  // one grid of boxes per mesh (the meshes of axia_gpu_setup_multi are
  // independent: no subdomain may hold nodes of two of them)
  const int nm = ctx->mesh_node0.size() >= 2 ? (int)ctx->mesh_node0.size() - 1 : 1;
  auto mesh_a0 = [&](int k) { return nm > 1 ? ctx->mesh_node0[k] : (int64_t)0; };
  auto mesh_a1 = [&](int k) { return nm > 1 ? ctx->mesh_node0[k + 1] : n; };
  const int max_boxes = COARSE_MAX / 6;
  std::vector<int64_t> target(nm);
  int64_t tsum = 0;
  for (int k = 0; k < nm; ++k) {
    target[k] = std::max<int64_t>(1, (mesh_a1(k) - mesh_a0(k)) / std::max(1, S->nodes_target));
    tsum += target[k];
  }
  if (!S->per_mesh) {
    if (tsum > max_boxes)
      for (int k = 0; k < nm; ++k) target[k] = std::max<int64_t>(1, target[k] * max_boxes / tsum);
  } else {
    // a block per mesh: at most max_boxes subdomains each, and the blocked
    // inversion (work ~ sum of block sizes cubed) at most twice that of one
    // 3072-unknown block
    const double budget = 2.0 * 3072.0 * 3072.0 * 3072.0;
    for (int k = 0; k < nm; ++k) target[k] = std::min<int64_t>(target[k], max_boxes);
    for (int it = 0; it < 200; ++it) {
      double work = 0.0;
      for (int k = 0; k < nm; ++k) work += std::pow(6.0 * (double)target[k], 3.0);
      if (work <= budget) break;
      for (int k = 0; k < nm; ++k) target[k] = std::max<int64_t>(1, (int64_t)(0.9 * (double)target[k]));
    }
  }
  std::vector<Grid3> grids(nm);
  std::vector<int> cell_base(nm + 1, 0);
  double* d_bb = nullptr;
  AXIA_TRY(dev_alloc(ctx, &d_bb, (size_t)6 * 1024));
  for (int k = 0; k < nm; ++k) {
    const int64_t nk = mesh_a1(k) - mesh_a0(k);
    const int bb_grid = (int)std::max<int64_t>(1, std::min<int64_t>((nk + 255) / 256, 1024));
    k_bbox<<<bb_grid, 256, 0, ctx->stream>>>(mesh_a0(k), mesh_a1(k), ctx->d_coords, d_bb);
    ctx->launches++;
    std::vector<double> hb((size_t)6 * bb_grid);
    const int cst = copy_to_host(ctx, hb.data(), d_bb, hb.size());
    if (cst) {
      dev_release(ctx, d_bb);
      return cst;
    }
    double lo[3] = {hb[0], hb[1], hb[2]}, hi[3] = {hb[3], hb[4], hb[5]};
    for (int b = 1; b < bb_grid; ++b)
      for (int d = 0; d < 3; ++d) {
        lo[d] = std::min(lo[d], hb[6 * b + d]);
        hi[d] = std::max(hi[d], hb[6 * b + 3 + d]);
      }
    double ext[3], emax = 0.0;
    for (int d = 0; d < 3; ++d) emax = std::max(emax, ext[d] = hi[d] - lo[d]);
    if (!(emax > 0.0) || !std::isfinite(emax)) emax = 1.0;
    double vol = 1.0;
    for (int d = 0; d < 3; ++d) vol *= std::max(ext[d], 1e-3 * emax);
    double h = std::cbrt(vol / (double)target[k]);
    Grid3 g{};
    for (int it = 0; it < 400; ++it) {
      g.nx = std::max(1, (int)std::ceil(ext[0] / h - 1e-9));
      g.ny = std::max(1, (int)std::ceil(ext[1] / h - 1e-9));
      g.nz = std::max(1, (int)std::ceil(ext[2] / h - 1e-9));
      if ((int64_t)g.nx * g.ny * g.nz <= target[k]) break;
      h *= 1.02;
    }
    if ((int64_t)g.nx * g.ny * g.nz > target[k]) {  // one box
      g.nx = g.ny = g.nz = 1;
      h = 2.0 * emax;
    }
    g.x0 = lo[0];
    g.y0 = lo[1];
    g.z0 = lo[2];
    g.h = h;
    grids[k] = g;
    cell_base[k + 1] = cell_base[k] + g.nx * g.ny * g.nz;
    if (k == 0) S->h = h;
  }
  dev_release(ctx, d_bb);
  const int ncell = cell_base[nm];
  if (!S->per_mesh && ncell > max_boxes + nm)
    return set_error(ctx, AXIA_ERR_TOO_LARGE, "coarse space: more than " + std::to_string(max_boxes) + " subdomains");
  int *d_cell = nullptr, *d_count = nullptr, *d_sub = nullptr, *d_iota = nullptr, *d_cellsub = nullptr;
  int* d_sub_sorted = nullptr;
  double *d_centre = nullptr, *d_inv_h = nullptr;
  unsigned char* d_temp = nullptr;  // cub scratch (pooled)
  int st = AXIA_OK;
  do {
    if ((st = dev_alloc(ctx, &d_cell, (size_t)n))) break;
    if ((st = dev_alloc(ctx, &d_count, (size_t)ncell))) break;
    AXIA_CUDA(ctx, cudaMemsetAsync(d_count, 0, ncell * sizeof(int), ctx->stream));
    for (int k = 0; k < nm; ++k) {
      k_cell_count<<<grid_for(ctx, mesh_a1(k) - mesh_a0(k), 256), 256, 0, ctx->stream>>>(
          mesh_a0(k), mesh_a1(k), ctx->d_coords, grids[k], cell_base[k], d_cell, d_count);
      ctx->launches++;
    }
    std::vector<int> count(ncell), cell_sub(ncell, -1);
    if ((st = copy_to_host(ctx, count.data(), d_count, (size_t)ncell))) break;
    int n_sub = 0;
    std::vector<int> sub_ptr(1, 0);
    std::vector<double> sub_inv_h;
    S->mesh_sub.assign(1, 0);
    for (int k = 0; k < nm; ++k) {
      for (int c = cell_base[k]; c < cell_base[k + 1]; ++c)
        if (count[c] > 0) {
          cell_sub[c] = n_sub++;
          sub_ptr.push_back(sub_ptr.back() + count[c]);
          sub_inv_h.push_back(1.0 / grids[k].h);
        }
      S->mesh_sub.push_back(n_sub);
    }
    // chunks of COARSE_CHUNK nodes inside every subdomain
    std::vector<int4> chunk;
    std::vector<int> chunk_ptr(1, 0);
    for (int I = 0; I < n_sub; ++I) {
      for (int b = sub_ptr[I]; b < sub_ptr[I + 1]; b += COARSE_CHUNK)
        chunk.push_back(make_int4(I, b, std::min(b + COARSE_CHUNK, sub_ptr[I + 1]), 0));
      chunk_ptr.push_back((int)chunk.size());
    }
    S->h_chunk_ptr = chunk_ptr;
    CoarseArgs& A = S->args;
    A.n_sub = n_sub;
    A.nc = 6 * n_sub;
    A.ncp = ((A.nc + GJ_T - 1) / GJ_T) * GJ_T;
    A.n_chunks = (int)chunk.size();
    A.row0 = 0;
    A.row1 = A.nc;
    A.chunk_lo = 0;
    A.chunk_hi = A.n_chunks;
    // diagonal blocks of the coarse matrix
    S->blk.clear();
    if (!S->per_mesh || nm == 1) {
      S->blk.push_back(CoarseBlk{0, A.nc, A.ncp, 0, 0});
    } else {
      long long off = 0;
      for (int k = 0; k < nm; ++k) {
        const int s0 = S->mesh_sub[k], ns = S->mesh_sub[k + 1] - s0;
        const int nk = 6 * ns, pk = std::max(GJ_T, ((nk + GJ_T - 1) / GJ_T) * GJ_T);
        S->blk.push_back(CoarseBlk{6 * s0, nk, pk, s0, off});
        off += (long long)pk * pk;
      }
    }
    S->blk_elems = 0;
    S->max_p = 0;
    int rc_len = A.ncp;
    std::vector<int> sub_blk(n_sub);
    for (int b = 0; b < (int)S->blk.size(); ++b) {
      const CoarseBlk& B = S->blk[b];
      S->blk_elems += (long long)B.p * B.p;
      S->max_p = std::max(S->max_p, B.p);
      rc_len = std::max(rc_len, B.u0 + B.p);
      for (int I = B.s0; I < B.s0 + B.n / 6; ++I) sub_blk[I] = b;
    }
    A.ncp = rc_len;  // length of the r_c / y buffers (one block: the padded size)
    A.col0 = 0;
    A.ldm = S->blk.size() == 1 ? S->blk[0].p : 0;  // per-mesh views set their own
    if ((st = dev_alloc(ctx, &S->d_blk, S->blk.size()))) break;
    if ((st = copy_to_device(ctx, S->d_blk, S->blk.data(), S->blk.size()))) break;
    if ((st = dev_alloc(ctx, &S->d_sub_blk, (size_t)n_sub))) break;
    if ((st = copy_to_device(ctx, S->d_sub_blk, sub_blk.data(), (size_t)n_sub))) break;
    if ((st = dev_alloc(ctx, &d_cellsub, (size_t)ncell))) break;
    if ((st = copy_to_device(ctx, d_cellsub, cell_sub.data(), (size_t)ncell))) break;
    if ((st = dev_alloc(ctx, &d_sub, (size_t)n))) break;
    if ((st = dev_alloc(ctx, &d_iota, (size_t)n))) break;
    if ((st = dev_alloc(ctx, &d_sub_sorted, (size_t)n))) break;
    if ((st = dev_alloc(ctx, &S->sub_node, (size_t)n))) break;
    k_sub_of_node<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(n, d_cell, d_cellsub, d_sub, d_iota);
    ctx->launches++;
    size_t temp_bytes = 0;
    int bits = 1;
    while ((1 << bits) < n_sub && bits < 30) ++bits;
    cub::DeviceRadixSort::SortPairs(nullptr, temp_bytes, d_sub, d_sub_sorted, d_iota, S->sub_node, (int)n, 0, bits,
                                    ctx->stream);
    if ((st = dev_alloc(ctx, &d_temp, std::max<size_t>(temp_bytes, 16)))) break;
    AXIA_CUDA(ctx, cub::DeviceRadixSort::SortPairs(d_temp, temp_bytes, d_sub, d_sub_sorted, d_iota, S->sub_node,
                                                   (int)n, 0, bits, ctx->stream));
    AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if ((st = dev_alloc(ctx, &S->sub_ptr, sub_ptr.size()))) break;
    if ((st = copy_to_device(ctx, S->sub_ptr, sub_ptr.data(), sub_ptr.size()))) break;
    if ((st = dev_alloc(ctx, &S->chunk, chunk.size()))) break;
    if ((st = copy_to_device(ctx, S->chunk, chunk.data(), chunk.size()))) break;
    if ((st = dev_alloc(ctx, &S->chunk_ptr, chunk_ptr.size()))) break;
    if ((st = copy_to_device(ctx, S->chunk_ptr, chunk_ptr.data(), chunk_ptr.size()))) break;
    if ((st = dev_alloc(ctx, &d_centre, (size_t)3 * n_sub))) break;
    if ((st = dev_alloc(ctx, &S->geo, (size_t)n))) break;
    if ((st = dev_alloc(ctx, &S->tmat, (size_t)36 * n_sub))) break;
    k_sub_centre<<<grid_for(ctx, (int64_t)n_sub * 32, 256), 256, 0, ctx->stream>>>(n_sub, S->sub_ptr, S->sub_node,
                                                                                  ctx->d_coords, d_centre);
    if ((st = dev_alloc(ctx, &d_inv_h, (size_t)n_sub))) break;
    if ((st = copy_to_device(ctx, d_inv_h, sub_inv_h.data(), (size_t)n_sub))) break;
    k_geo<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(n, ctx->d_coords, d_sub, d_centre, d_inv_h, ctx->d_ind_of,
                                                          S->geo);
    k_sub_gram<<<grid_for(ctx, (int64_t)n_sub * 32, 128), 128, 0, ctx->stream>>>(n_sub, S->sub_ptr, S->sub_node,
                                                                                S->geo, S->tmat);
    ctx->launches += 3;
    AXIA_CUDA(ctx, cudaGetLastError());
    if ((st = dev_alloc(ctx, &S->part, (size_t)6 * A.n_chunks))) break;
    if ((st = dev_alloc(ctx, &S->yc, (size_t)A.ncp))) break;
    if ((st = dev_alloc(ctx, &S->rc, (size_t)A.ncp))) break;
    if ((st = dev_alloc(ctx, &S->cnt, (size_t)n_sub))) break;
    AXIA_CUDA(ctx, cudaMemsetAsync(S->rc, 0, A.ncp * sizeof(float), ctx->stream));
    if ((st = dev_alloc(ctx, &S->minv, (size_t)S->blk_elems))) break;
    AXIA_CUDA(ctx, cudaMemsetAsync(S->yc, 0, A.ncp * sizeof(float), ctx->stream));
    AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    A.sub_node = S->sub_node;
    A.chunk = S->chunk;
    A.chunk_ptr = S->chunk_ptr;
    A.geo = S->geo;
    A.minv = S->minv;
    A.part = S->part;
    A.rc = S->rc;
    A.cnt = S->cnt;
    A.yc = S->yc;
  } while (false);
  dev_release(ctx, d_temp);
  dev_release(ctx, d_cell);
  dev_release(ctx, d_count);
  dev_release(ctx, d_sub);
  dev_release(ctx, d_iota);
  dev_release(ctx, d_cellsub);
  dev_release(ctx, d_sub_sorted);
  dev_release(ctx, d_centre);
  dev_release(ctx, d_inv_h);
  return st;
}

__global__ void k_iota(int n, int* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = i;
}

// the items of every node row from the FP32 node-block matrix when it is
// assembled, else from the FP64 one
void launch_row_items(axia_ctx* ctx, int n, int n_sub, const float4* geo, CoarseState* S) {
  const unsigned grid = grid_for(ctx, (int64_t)n * 32, 32 * ROW_WARPS);
  if (ctx->have_bsr32) {
    const BsrMat<float> K{(int)ctx->n_nodes, ctx->d_qptr, ctx->d_qadj, ctx->d_bval32, (long long)ctx->nbq};
    k_row_items<float><<<grid, 32 * ROW_WARPS, 0, ctx->stream>>>(n, n_sub, K, geo, S->off, S->keys, S->vals);
  } else {
    const BsrMat<double> K{(int)ctx->n_nodes, ctx->d_qptr, ctx->d_qadj, ctx->d_bval64, (long long)ctx->nbq};
    k_row_items<double><<<grid, 32 * ROW_WARPS, 0, ctx->stream>>>(n, n_sub, K, geo, S->off, S->keys, S->vals);
  }
  ctx->launches++;
}

// Items of the node rows and their runs: they depend on the subdomains and
// the constraints only, so they are built once per space.
int build_item_structure(axia_ctx* ctx, CoarseState* S) {
  CoarseArgs& A = S->args;
  const int n = (int)ctx->n_nodes, n_sub = A.n_sub;
  int *d_cnt = nullptr, *d_iota = nullptr, *d_nruns = nullptr;
  unsigned* d_keys_sorted = nullptr;
  unsigned char* d_temp = nullptr;  // cub scratch (pooled)
  int st = AXIA_OK;
  do {
    if ((st = reset_dev_status(ctx))) break;
    if ((st = dev_alloc(ctx, &d_cnt, (size_t)n + 1))) break;
    if ((st = dev_alloc(ctx, &S->off, (size_t)n + 1))) break;
    AXIA_CUDA(ctx, cudaMemsetAsync(d_cnt + n, 0, sizeof(int), ctx->stream));
    k_row_count<<<grid_for(ctx, (int64_t)n * 32, 256), 256, 0, ctx->stream>>>(n, ctx->d_qptr, ctx->d_qadj, A.geo,
                                                                             d_cnt, ctx->d_status);
    ctx->launches++;
    if ((st = read_status(ctx, "a node row touches more than 32 subdomains (raise coarse_nodes)"))) break;
    size_t tb = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tb, d_cnt, S->off, n + 1, ctx->stream);
    if ((st = dev_alloc(ctx, &d_temp, std::max<size_t>(tb, 16)))) break;
    AXIA_CUDA(ctx, cub::DeviceScan::ExclusiveSum(d_temp, tb, d_cnt, S->off, n + 1, ctx->stream));
    if ((st = copy_to_host(ctx, &S->n_items, S->off + n, 1))) break;
    dev_release(ctx, d_temp);
    const int ni = std::max(S->n_items, 1);
    if ((st = dev_alloc(ctx, &S->keys, (size_t)ni))) break;
    if ((st = dev_alloc(ctx, &d_keys_sorted, (size_t)ni))) break;
    if ((st = dev_alloc(ctx, &S->vals, (size_t)ni * 36))) break;
    if ((st = dev_alloc(ctx, &d_iota, (size_t)ni))) break;
    if ((st = dev_alloc(ctx, &S->perm, (size_t)ni))) break;
    launch_row_items(ctx, n, n_sub, A.geo, S);
    AXIA_CUDA(ctx, cudaGetLastError());
    k_iota<<<grid_for(ctx, ni, 256), 256, 0, ctx->stream>>>(ni, d_iota);
    ctx->launches++;
    int bits = 1;
    while ((1ull << bits) < (unsigned long long)n_sub * n_sub && bits < 32) ++bits;
    cub::DeviceRadixSort::SortPairs(nullptr, tb, S->keys, d_keys_sorted, d_iota, S->perm, S->n_items, 0, bits,
                                    ctx->stream);
    if ((st = dev_alloc(ctx, &d_temp, std::max<size_t>(tb, 16)))) break;
    AXIA_CUDA(ctx, cub::DeviceRadixSort::SortPairs(d_temp, tb, S->keys, d_keys_sorted, d_iota, S->perm, S->n_items,
                                                   0, bits, ctx->stream));
    AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    dev_release(ctx, d_temp);
    if ((st = dev_alloc(ctx, &S->run_key, (size_t)ni))) break;
    if ((st = dev_alloc(ctx, &S->run_cnt, (size_t)ni))) break;
    if ((st = dev_alloc(ctx, &S->run_off, (size_t)ni))) break;
    if ((st = dev_alloc(ctx, &d_nruns, 1))) break;
    cub::DeviceRunLengthEncode::Encode(nullptr, tb, d_keys_sorted, S->run_key, S->run_cnt, d_nruns, S->n_items,
                                       ctx->stream);
    if ((st = dev_alloc(ctx, &d_temp, std::max<size_t>(tb, 16)))) break;
    AXIA_CUDA(ctx, cub::DeviceRunLengthEncode::Encode(d_temp, tb, d_keys_sorted, S->run_key, S->run_cnt, d_nruns,
                                                      S->n_items, ctx->stream));
    if ((st = copy_to_host(ctx, &S->n_runs, d_nruns, 1))) break;
    dev_release(ctx, d_temp);
    cub::DeviceScan::ExclusiveSum(nullptr, tb, S->run_cnt, S->run_off, S->n_runs, ctx->stream);
    if ((st = dev_alloc(ctx, &d_temp, std::max<size_t>(tb, 16)))) break;
    AXIA_CUDA(ctx, cub::DeviceScan::ExclusiveSum(d_temp, tb, S->run_cnt, S->run_off, S->n_runs, ctx->stream));
    AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const size_t ncp = (size_t)A.ncp;
    if ((st = dev_alloc(ctx, &S->a64, (size_t)S->blk_elems))) break;
    if ((st = dev_alloc(ctx, &S->a32, (size_t)S->blk_elems))) break;
    if ((st = dev_alloc(ctx, &S->scale, ncp))) break;
    if ((st = dev_alloc(ctx, &S->piv, (size_t)GJ_GROUPS * 2 * GJ_T * GJ_T))) break;
    if ((st = dev_alloc(ctx, &S->gj_bar, (size_t)GJ_GROUPS))) break;
    S->items_fresh = true;  // the values of this pass belong to the current K
  } while (false);
  dev_release(ctx, d_temp);
  dev_release(ctx, d_cnt);
  dev_release(ctx, d_iota);
  dev_release(ctx, d_nruns);
  dev_release(ctx, d_keys_sorted);
  return st;
}

// s_i = 1 / sqrt(A_ii) for the coarse unknowns whose diagonal is positive
// (above 1e-12 of the largest), 0 for the rest and the padding (one block)
// diagonal entry of unknown i (its subdomain's block)
__device__ __forceinline__ double coarse_diag(const double* A, const CoarseBlk* blk, const int* sub_blk, int i) {
  const CoarseBlk K = blk[sub_blk[i / 6]];
  return A[K.off + (size_t)(i - K.u0) * (K.p + 1)];
}

__global__ void k_diag_scale(int nc, int ncp, const double* A, const CoarseBlk* blk, const int* sub_blk,
                             double* scale) {
  __shared__ double red[32];
  double m = 0.0;
  for (int i = threadIdx.x; i < nc; i += blockDim.x) {
    const double d = coarse_diag(A, blk, sub_blk, i);
    if (isfinite(d)) m = fmax(m, d);
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) red[0] = m;
  }
  __syncthreads();
  const double dmax = red[0];
  for (int i = threadIdx.x; i < ncp; i += blockDim.x) {
    const double d = i < nc ? coarse_diag(A, blk, sub_blk, i) : 0.0;
    scale[i] = (i < nc && isfinite(d) && d > 1e-12 * dmax) ? 1.0 / sqrt(d) : 0.0;
  }
}

// coarse operator and its inverse from the assembled FP64 node-block matrix
int build_operator(axia_ctx* ctx, CoarseState* S) {
  CoarseArgs& A = S->args;
  const int n = (int)ctx->n_nodes, n_sub = A.n_sub, nc = A.nc, ncp = A.ncp;
  if (!S->off) AXIA_TRY(build_item_structure(ctx, S));
  if (!S->items_fresh) launch_row_items(ctx, n, n_sub, A.geo, S);
  S->items_fresh = false;
  const int nblk = (int)S->blk.size();
  if (nblk > 65535) return set_error(ctx, AXIA_ERR_TOO_LARGE, "coarse space: more than 65535 meshes");
  AXIA_CUDA(ctx, cudaMemsetAsync(S->a64, 0, (size_t)S->blk_elems * sizeof(double), ctx->stream));
  k_run_sum<<<grid_for(ctx, (int64_t)S->n_runs * 32, 256), 256, 0, ctx->stream>>>(
      S->n_runs, n_sub, S->run_key, S->run_off, S->run_cnt, S->perm, S->vals, S->tmat, S->a64, S->d_blk,
      S->d_sub_blk);
  // unit-diagonal scaling; modes without stiffness (dropped or padding) become identity
  k_diag_scale<<<1, 1024, 0, ctx->stream>>>(nc, ncp, S->a64, S->d_blk, S->d_sub_blk, S->scale);
  {
    const int gx = grid_for(ctx, (int64_t)S->max_p * S->max_p, 256);
    k_scale_to_f32<<<dim3((unsigned)std::max(1, gx / std::max(1, std::min(nblk, 16))), (unsigned)nblk), 256, 0,
                     ctx->stream>>>(S->d_blk, S->a64, S->scale, S->a32);
  }
  ctx->launches += 3;
  AXIA_CUDA(ctx, cudaGetLastError());
  AXIA_TRY(reset_dev_status(ctx));
  {
    int per_sm = 0;
    AXIA_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gj_inverse, GJ_THREADS, 0));
    if (per_sm < 1) return set_error(ctx, AXIA_ERR_CUDA, "coarse space: inverse kernel does not fit");
    const int nt = S->max_p / GJ_T;
    const int full = std::min(per_sm, 2) * ctx->sm_count;
    int grid = std::max(2, std::min(full, std::max(2, nt * (nt - 1) / 2)));
    // several blocks: groups of at least 16 launch blocks invert them side by side
    int ngroups = 1;
    if (nblk > 1) {
      grid = std::max(2, full);
      ngroups = std::max(1, std::min(std::min(nblk, GJ_GROUPS), grid / 16));
    }
    AXIA_CUDA(ctx, cudaMemsetAsync(S->gj_bar, 0, sizeof(GridBarrier) * GJ_GROUPS, ctx->stream));
    GjArgs P{S->a32, S->max_p, S->piv, S->gj_bar, ctx->d_status, 2000000000ull, 0, grid};
    const CoarseBlk* dblk = S->d_blk;
    void* params[] = {&P, &dblk, (void*)&nblk, &ngroups};
    AXIA_CUDA(ctx, cudaLaunchCooperativeKernel((const void*)k_gj_inverse, dim3(grid), dim3(GJ_THREADS), params, 0,
                                               ctx->stream));
    ctx->launches++;
  }
  AXIA_CUDA(ctx, cudaMemsetAsync(S->minv, 0, (size_t)S->blk_elems * sizeof(float), ctx->stream));
  {
    int max_ns = 0;
    for (const CoarseBlk& B : S->blk) max_ns = std::max(max_ns, B.n / 6);
    const int gx = grid_for(ctx, (int64_t)max_ns * max_ns, 128);
    k_minv<<<dim3((unsigned)std::max(1, gx / std::max(1, std::min(nblk, 16))), (unsigned)nblk), 128, 0,
             ctx->stream>>>(S->d_blk, S->a32, S->scale, S->tmat, S->minv);
  }
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  return read_status(ctx, "coarse operator is not positive definite");
}

}  // namespace

void coarse_release(axia_ctx* ctx) {
  auto* S = static_cast<CoarseState*>(ctx->coarse);
  if (!S) return;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  S->release(ctx);
  delete S;
  ctx->coarse = nullptr;
}

// The coarse space of the current mesh (built on first use, or when the
// requested subdomain size changes) and its operator for the current
// assembly (rebuilt after every assembly).
// Default subdomain size: about 512 subdomains (8^3 for a cube; the dense
// inverse then costs about 4 ms), but no fewer than about 13,500 matrix node
// blocks per subdomain -- 500 nodes for C3D8 (27 blocks per node row), about
// 250 for C3D20 (about 55).  Measured per step: C3D20 50^3 350 iterations
// and 147 ms with 216 subdomains, 271 and 127 ms with 512; SIMP C3D8
// 100x50x50 236 iterations and 31.1 ms with 125 subdomains, 167 and 26.9 ms
// with 512; the C3D8 100^3 headline keeps its 512.
static int default_nodes_target(const axia_ctx* ctx) {
  if (ctx->n_adj <= 0 || ctx->n_nodes <= 0) return 2000;
  const double floor_nodes = 500.0 * 27.0 * (double)ctx->n_nodes / (double)ctx->n_adj;
  const double v = std::max(floor_nodes, (double)ctx->n_nodes / 512.0);
  return (int)std::min(1.0e6, std::max(16.0, v));
}

int coarse_prepare(axia_ctx* ctx, int nodes_target, CoarseArgs* out, bool per_mesh) {
  if (!ctx->have_bsr64) return set_error(ctx, AXIA_ERR_STATE, "coarse space needs the FP64 node-block matrix");
  if (nodes_target <= 0) nodes_target = default_nodes_target(ctx);
  per_mesh = per_mesh && ctx->mesh_node0.size() >= 3;  // two or more meshes
  auto* S = static_cast<CoarseState*>(ctx->coarse);
  if (S && (S->nodes_target != nodes_target || S->per_mesh != per_mesh)) {
    coarse_release(ctx);
    S = nullptr;
  }
  if (!S) {
    S = new CoarseState();
    S->nodes_target = nodes_target;
    S->per_mesh = per_mesh;
    ++ctx->coarse_gen;
    ctx->coarse = S;
    const int st = build_space(ctx, S);
    if (st) {
      coarse_release(ctx);
      return st;
    }
  }
  if (S->op_gen != ctx->assemble_gen) {
    AXIA_TRY(build_operator(ctx, S));
    S->op_gen = ctx->assemble_gen;
  }
  // arrival counters of the restriction (a stopped solve may leave them set)
  AXIA_CUDA(ctx, cudaMemsetAsync(S->cnt, 0, (size_t)S->args.n_sub * sizeof(int), ctx->stream));
  *out = S->args;
  return AXIA_OK;
}

// The same, plus the 32-column buffers of the batched solve.
int coarse_prepare_batched(axia_ctx* ctx, int nodes_target, CoarseArgs* out) {
  AXIA_TRY(coarse_prepare(ctx, nodes_target, out));
  auto* S = static_cast<CoarseState*>(ctx->coarse);
  if (!S->part_m) {
    AXIA_TRY(dev_alloc(ctx, &S->part_m, (size_t)S->args.n_chunks * 6 * 32));
    AXIA_TRY(dev_alloc(ctx, &S->rc_m, (size_t)S->args.ncp * 32));
    AXIA_TRY(dev_alloc(ctx, &S->yc_m, (size_t)S->args.ncp * 32));
    AXIA_CUDA(ctx, cudaMemsetAsync(S->rc_m, 0, (size_t)S->args.ncp * 32 * sizeof(float), ctx->stream));
    AXIA_CUDA(ctx, cudaMemsetAsync(S->yc_m, 0, (size_t)S->args.ncp * 32 * sizeof(float), ctx->stream));
    S->args.part_m = S->part_m;
    S->args.rc_m = S->rc_m;
    S->args.yc_m = S->yc_m;
  }
  *out = S->args;
  return AXIA_OK;
}

// per mesh of a multi-mesh context: its restriction chunks and coarse rows
int coarse_mesh_ranges(const axia_ctx* ctx, std::vector<int>& chunk0, std::vector<int>& chunk1, std::vector<int>& row0,
                       std::vector<int>& row1, std::vector<int>& col0, std::vector<int>& ldm,
                       std::vector<long long>& moff) {
  const auto* S = static_cast<const CoarseState*>(ctx->coarse);
  if (!S) return AXIA_ERR_STATE;
  const int nm = (int)S->mesh_sub.size() - 1;
  chunk0.resize(nm);
  chunk1.resize(nm);
  row0.resize(nm);
  row1.resize(nm);
  col0.resize(nm);
  ldm.resize(nm);
  moff.resize(nm);
  for (int k = 0; k < nm; ++k) {
    chunk0[k] = S->h_chunk_ptr[S->mesh_sub[k]];
    chunk1[k] = S->h_chunk_ptr[S->mesh_sub[k + 1]];
    row0[k] = 6 * S->mesh_sub[k];
    row1[k] = 6 * S->mesh_sub[k + 1];
    // one block for all meshes: every mesh reads it whole (col0 = 0)
    const CoarseBlk& B = S->blk.size() == (size_t)nm ? S->blk[k] : S->blk[0];
    col0[k] = B.u0;
    ldm[k] = B.p;
    moff[k] = B.off;
  }
  return AXIA_OK;
}

extern "C" int32_t axia_gpu_coarse_size(const axia_ctx* ctx, int64_t* n_sub, int64_t* n_coarse) {
  if (!ctx || !n_sub || !n_coarse) return AXIA_ERR_INVALID_ARG;
  const auto* S = static_cast<const CoarseState*>(ctx->coarse);
  *n_sub = S ? S->args.n_sub : 0;
  *n_coarse = S ? S->args.nc : 0;
  return AXIA_OK;
}
