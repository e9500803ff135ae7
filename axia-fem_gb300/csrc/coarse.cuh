// coarse.cuh -- the coarse space of the two-level preconditioner of the mixed
// node-block solve (device side, used inside the persistent CG kernel).
//
// No reference counterpart: the reference preconditions its CG with the
// diagonal only (solver/src/linalg.rs:199-259).  The solution it converges to
// is the same; only the iteration count changes.
//
// The mesh nodes are split into subdomains (cells of a uniform grid over the
// bounding box).  Each subdomain I contributes the six rigid-body modes of its
// nodes -- three translations and three rotations about its centre c_I --
// restricted to the free DOFs: for node a with r = (x_a - c_I) / h,
//   Z_a = [ e_x  e_y  e_z  (0, -r_z, r_y)  (r_z, 0, -r_x)  (-r_y, r_x, 0) ],
// with the rows of prescribed DOFs zero.  The preconditioner is additive,
//   z = D^-1 r + Z M Z^T r ,   M = (Z^T K Z)^+ ,
// M in the raw mode basis (the per-subdomain orthonormalisation and the
// dropped modes folded in at setup).  Per CG iteration that is three phases:
//   restrict  inside the x / r update, which runs node by node over fixed
//             chunks of each subdomain's node list: partials of Z^T r per
//             chunk, summed in chunk order by the warp that finishes a
//             subdomain's last chunk (after an FP64 residual replaced r, a
//             separate pass does the same)
//   solve     every block copies r_c to shared memory, warps take rows of
//             y = M r_c, and r_c . y = r . Z y (the coarse part of r . z) goes
//             into a partial-sum slot
//   prolong   inside the search-direction update, one node per thread:
//             p = D^-1 r + Z y + beta p
// All sums run in a fixed order, so the solve stays bitwise reproducible.
#pragma once

#include "solver.cuh"

// The coarse-space constants and CoarseArgs live in solver.cuh (they are
// part of the solver's argument pack).

// Builds (or reuses) the coarse space of the current mesh and its operator
// for the current assembly (coarse.cu); nodes_target <= 0: about 512
// subdomains, at least about 13,500 node blocks each (500 nodes for C3D8).
// per_mesh (multi-mesh solve): a block of the coarse inverse per mesh, so
// every mesh may have as many subdomains as one mesh alone.
int coarse_prepare(axia_ctx* ctx, int nodes_target, CoarseArgs* out, bool per_mesh = false);
// The same with the 32-column buffers of the batched load-case solve.
int coarse_prepare_batched(axia_ctx* ctx, int nodes_target, CoarseArgs* out);
// Per mesh of a multi-mesh context: its restriction chunks, coarse rows and
// block of the coarse inverse (padded size, element offset).
int coarse_mesh_ranges(const axia_ctx* ctx, std::vector<int>& chunk0, std::vector<int>& chunk1,
                       std::vector<int>& row0, std::vector<int>& row1, std::vector<int>& col0,
                       std::vector<int>& ldm, std::vector<long long>& moff);

__device__ __forceinline__ unsigned geo_bits(float4 g) { return __float_as_uint(g.w); }

// Z_a^T r_a of one node added to v (r masked by the node's free DOFs)
__device__ __forceinline__ void zt_add(float4 g, float rx, float ry, float rz, float (&v)[6]) {
  v[0] += rx;
  v[1] += ry;
  v[2] += rz;
  v[3] = fmaf(g.y, rz, fmaf(-g.z, ry, v[3]));
  v[4] = fmaf(g.z, rx, fmaf(-g.x, rz, v[4]));
  v[5] = fmaf(g.x, ry, fmaf(-g.y, rx, v[5]));
}

// Chunk c of subdomain I is done: its six sums go to part[c]; the warp that
// finishes the last chunk of I adds the chunk sums in chunk order (the same
// bits whichever warp that is) into r_c[6 I ..] and re-arms the counter.
__device__ __forceinline__ void coarse_chunk_finish(const CoarseArgs& C, int c, int I, float (&v)[6], int lane) {
#pragma unroll
  for (int k = 0; k < 6; ++k) v[k] = warp_sum(v[k]);
  if (lane < 6) {
    const float x = lane == 0 ? v[0] : lane == 1 ? v[1] : lane == 2 ? v[2] : lane == 3 ? v[3] : lane == 4 ? v[4] : v[5];
    C.part[6 * c + lane] = x;
  }
  __threadfence();
  __syncwarp();
  const int c0 = __ldg(C.chunk_ptr + I), c1 = __ldg(C.chunk_ptr + I + 1);
  int last = 0;
  if (lane == 0) last = atomicAdd(C.cnt + I, 1) == c1 - c0 - 1;
  last = __shfl_sync(0xffffffffu, last, 0);
  if (last) {
    __threadfence();
    if (lane < 6) C.rc[6 * I + lane] = ldcg_sum(C.part + 6 * c0 + lane, 6, c1 - c0);
    if (lane == 0) atomicExch(C.cnt + I, 0);
  }
}

// r_c = Z^T r over the chunks (after an FP64 residual replaced r, and at the start)
__device__ __forceinline__ void coarse_restrict(const CoarseArgs& C, const float* r, int gwarp, int nwarps,
                                                int lane) {
  for (int c = C.chunk_lo + gwarp; c < C.chunk_hi; c += nwarps) {
    const int4 ch = C.chunk[c];
    float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll 4
    for (int k = ch.y + lane; k < ch.z; k += 32) {
      const int a = __ldg(C.sub_node + k);
      const float4 g = __ldg(C.geo + a);
      const unsigned m = geo_bits(g);
      zt_add(g, (m & 1u) ? r[3 * a] : 0.f, (m & 2u) ? r[3 * a + 1] : 0.f, (m & 4u) ? r[3 * a + 2] : 0.f, v);
    }
    coarse_chunk_finish(C, c, ch.x, v, lane);
  }
}

// The CG update x += alpha p, r -= alpha q node by node in subdomain order,
// with the partial sums of r.r and r.D^-1 r and the restriction of the new r.
__device__ __forceinline__ void coarse_update_restrict(const CoarseArgs& C, float alpha, float* x, const float* p,
                                                       const float* q, float* r, const float* dinv, int gwarp,
                                                       int nwarps, int lane, float& rr_p, float& rz_p) {
  for (int c = C.chunk_lo + gwarp; c < C.chunk_hi; c += nwarps) {
    const int4 ch = C.chunk[c];
    float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll 4
    for (int k = ch.y + lane; k < ch.z; k += 32) {
      const int a = __ldg(C.sub_node + k);
      const float4 g = __ldg(C.geo + a);
      const unsigned m = geo_bits(g);
      float rv[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const int i = 3 * a + d;
        x[i] = fmaf(alpha, p[i], x[i]);
        const float ri = fmaf(-alpha, q[i], r[i]);
        r[i] = ri;
        rr_p = fmaf(ri, ri, rr_p);
        rz_p = fmaf(ri, ri * dinv[i], rz_p);
        rv[d] = ((m >> d) & 1u) ? ri : 0.f;
      }
      zt_add(g, rv[0], rv[1], rv[2], v);
    }
    coarse_chunk_finish(C, c, ch.x, v, lane);
  }
}

// The block's part of r_c into shared memory (zero past its unknowns), then
// rows of y = M r_c over the warps of the group.  Returns this thread's share
// of r_c . y (nonzero on lane 0 of warps that own rows).
__device__ __forceinline__ float coarse_solve(const CoarseArgs& C, float* s_rc, int gwarp, int nwarps, int lane) {
  if (C.col0 == 0 && C.row0 == 0 && C.row1 == C.nc && C.ldm <= C.ncp) {  // the whole matrix: r_c is zero past nc
    for (int t = threadIdx.x; t < (C.ldm >> 2); t += blockDim.x)
      reinterpret_cast<float4*>(s_rc)[t] = __ldcg(reinterpret_cast<const float4*>(C.rc) + t);
  } else {
    for (int t = threadIdx.x; t < C.ldm; t += blockDim.x) s_rc[t] = C.col0 + t < C.row1 ? __ldcg(C.rc + C.col0 + t) : 0.f;
  }
  __syncthreads();
  float acc = 0.f;
  const int nq = C.ldm >> 2;
  const float4* rc4 = reinterpret_cast<const float4*>(s_rc);
  for (int row = C.row0 + gwarp; row < C.row1; row += nwarps) {
    const float4* m = reinterpret_cast<const float4*>(C.minv + (size_t)(row - C.col0) * C.ldm);
    float s = 0.f;
#pragma unroll 4
    for (int j = lane; j < nq; j += 32) {
      const float4 mv = __ldcs(m + j);  // streamed: M must not push the CG vectors out of L2
      const float4 rv = rc4[j];
      s = fmaf(mv.x, rv.x, fmaf(mv.y, rv.y, fmaf(mv.z, rv.z, fmaf(mv.w, rv.w, s))));
    }
    s = warp_sum(s);
    if (lane == 0) {
      C.yc[row] = s;
      acc = fmaf(s, s_rc[row - C.col0], acc);
    }
  }
  return acc;
}

// p = D^-1 r + Z y + beta p over the nodes [n0, n1): one geo load and the
// subdomain's six y per node, then its three DOFs (beta = 0, add = true: p += Z y).
__device__ __forceinline__ void coarse_update_p(const CoarseArgs& C, int n0, int n1, int tid, int nth, float beta,
                                                const float* r, const float* dinv, float* p, bool add_only) {
#pragma unroll 2
  for (int a = n0 + tid; a < n1; a += nth) {
    const float4 g = __ldg(C.geo + a);
    const unsigned m = geo_bits(g);
    const float* y = C.yc + 6 * (m >> 3);
    const float y0 = y[0], y1 = y[1], y2 = y[2], y3 = y[3], y4 = y[4], y5 = y[5];
    const float zc[3] = {(m & 1u) ? fmaf(g.z, y4, fmaf(-g.y, y5, y0)) : 0.f,
                         (m & 2u) ? fmaf(-g.z, y3, fmaf(g.x, y5, y1)) : 0.f,
                         (m & 4u) ? fmaf(g.y, y3, fmaf(-g.x, y4, y2)) : 0.f};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int i = 3 * a + c;
      if (add_only)
        p[i] += zc[c];
      else
        p[i] = fmaf(beta, p[i], fmaf(r[i], dinv[i], zc[c]));
    }
  }
}
