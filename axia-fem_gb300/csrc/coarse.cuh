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
//   restrict  partials of Z^T r over fixed chunks of each subdomain's node list
//   solve     every block sums the partials into r_c (shared memory, fixed
//             order), warps take rows of y = M r_c, and r_c . y = r . Z y
//             (the coarse part of r . z) goes into a partial-sum slot
//   prolong   inside the search-direction update, one node per thread:
//             p = D^-1 r + Z y + beta p
// All sums run in a fixed order, so the solve stays bitwise reproducible.
#pragma once

#include "solver.cuh"

// The coarse-space constants and CoarseArgs live in solver.cuh (they are
// part of the solver's argument pack).

// Builds (or reuses) the coarse space of the current mesh and its operator
// for the current assembly (coarse.cu); nodes_target <= 0: 2000.
int coarse_prepare(axia_ctx* ctx, int nodes_target, CoarseArgs* out);

__device__ __forceinline__ unsigned geo_bits(float4 g) { return __float_as_uint(g.w); }

// Restriction partials: chunk c of subdomain I gets sum over its nodes of Z_a^T r_a.
__device__ __forceinline__ void coarse_restrict(const CoarseArgs& C, const float* r, int gwarp, int nwarps,
                                                int lane) {
  for (int c = gwarp; c < C.n_chunks; c += nwarps) {
    const int4 ch = C.chunk[c];
    float v0 = 0.f, v1 = 0.f, v2 = 0.f, v3 = 0.f, v4 = 0.f, v5 = 0.f;
#pragma unroll 4
    for (int k = ch.y + lane; k < ch.z; k += 32) {
      const int a = __ldg(C.sub_node + k);
      const float4 g = __ldg(C.geo + a);
      const unsigned m = geo_bits(g);
      const float rx = (m & 1u) ? r[3 * a] : 0.f;
      const float ry = (m & 2u) ? r[3 * a + 1] : 0.f;
      const float rz = (m & 4u) ? r[3 * a + 2] : 0.f;
      v0 += rx;
      v1 += ry;
      v2 += rz;
      v3 = fmaf(g.y, rz, fmaf(-g.z, ry, v3));
      v4 = fmaf(g.z, rx, fmaf(-g.x, rz, v4));
      v5 = fmaf(g.x, ry, fmaf(-g.y, rx, v5));
    }
    v0 = warp_sum(v0);
    v1 = warp_sum(v1);
    v2 = warp_sum(v2);
    v3 = warp_sum(v3);
    v4 = warp_sum(v4);
    v5 = warp_sum(v5);
    if (lane < 6) {
      const float v = lane == 0 ? v0 : lane == 1 ? v1 : lane == 2 ? v2 : lane == 3 ? v3 : lane == 4 ? v4 : v5;
      C.part[6 * c + lane] = v;
    }
  }
}

// r_c into shared memory (every block the same sums in the same order), then
// rows of y = M r_c over the warps of the group.  Returns this thread's share
// of r_c . y (nonzero on lane 0 of warps that own rows).
__device__ __forceinline__ float coarse_solve(const CoarseArgs& C, float* s_rc, int gwarp, int nwarps, int lane) {
  for (int t = threadIdx.x; t < C.ncp; t += blockDim.x) {
    float s = 0.f;
    if (t < C.nc) {
      const int I = t / 6, i = t - 6 * I;
      const int c1 = __ldg(C.chunk_ptr + I + 1);
#pragma unroll 4
      for (int c = __ldg(C.chunk_ptr + I); c < c1; ++c) s += C.part[6 * c + i];
    }
    s_rc[t] = s;
  }
  __syncthreads();
  float acc = 0.f;
  const int nq = C.ncp >> 2;
  const float4* rc4 = reinterpret_cast<const float4*>(s_rc);
  for (int row = gwarp; row < C.nc; row += nwarps) {
    const float4* m = reinterpret_cast<const float4*>(C.minv + (size_t)row * C.ncp);
    float s = 0.f;
#pragma unroll 4
    for (int j = lane; j < nq; j += 32) {
      const float4 mv = __ldg(m + j);
      const float4 rv = rc4[j];
      s = fmaf(mv.x, rv.x, fmaf(mv.y, rv.y, fmaf(mv.z, rv.z, fmaf(mv.w, rv.w, s))));
    }
    s = warp_sum(s);
    if (lane == 0) {
      C.yc[row] = s;
      acc = fmaf(s, s_rc[row], acc);
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
