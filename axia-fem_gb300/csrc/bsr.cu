// bsr.cu -- the node-block (3x3 BSR) form of the static system and the
// persistent Krylov kernels on it.
//
// Layout: one block row per node a, one 3x3 block per adjacent node b (the
// node adjacency of the symbolic phase, sorted), each block row padded with
// zero blocks to a multiple of 4 blocks; values stored as nine
// structure-of-arrays planes val[k][s] (k = 3 i + j).  A lane loads VEC = 1,
// 2 or 4 consecutive blocks of its row with one vector load per plane (and
// one for their block columns), so a warp has 4 to 16 times the bytes of a
// one-block-per-lane loop in flight: the SpMV is bound by DRAM latency
// unless each lane keeps enough loads outstanding.  Index traffic is one
// int32 per 9 values: 4.44 bytes per nonzero in FP32 (CSR: 8) and 8.44 in
// FP64 (CSR: 12), plus the padding (C3D8 interior rows: 27 -> 28 blocks).
//
// The system is the full-DOF form of K_ff: rows and columns of prescribed
// DOFs are zero except a unit diagonal, their right-hand side is zero.  CG on
// it produces the same iterates as CG on K_ff (the prescribed components of
// r, z, p, q, x stay exactly zero) with vectors of 3 n_nodes entries, so the
// DOF map never enters the inner loop.
//
// Kernels: bsr_spmv_kernel (y = K x), pcg_bsr_kernel (Jacobi PCG as in
// solver/src/linalg.rs:199-259, FP64 or FP32) and pcg_bsr_reliable_kernel
// (FP32 inner CG with FP64 reliable updates, the mixed form).
#include <algorithm>
#include <string>
#include <cstdlib>
#include <cstdio>
#include <type_traits>
#include <vector>
#include <cmath>

#include "coarse.cuh"

// Vector loads of VEC consecutive entries (streaming: the matrix is read once per use).
template <typename V, int VEC>
__device__ __forceinline__ void ldv(const V* p, V (&o)[VEC]);
template <>
__device__ __forceinline__ void ldv<float, 1>(const float* p, float (&o)[1]) { o[0] = __ldcs(p); }
template <>
__device__ __forceinline__ void ldv<float, 2>(const float* p, float (&o)[2]) {
  const float2 t = __ldcs(reinterpret_cast<const float2*>(p));
  o[0] = t.x;
  o[1] = t.y;
}
template <>
__device__ __forceinline__ void ldv<float, 4>(const float* p, float (&o)[4]) {
  const float4 t = __ldcs(reinterpret_cast<const float4*>(p));
  o[0] = t.x;
  o[1] = t.y;
  o[2] = t.z;
  o[3] = t.w;
}
template <>
__device__ __forceinline__ void ldv<double, 1>(const double* p, double (&o)[1]) { o[0] = __ldcs(p); }
template <>
__device__ __forceinline__ void ldv<double, 2>(const double* p, double (&o)[2]) {
  const double2 t = __ldcs(reinterpret_cast<const double2*>(p));
  o[0] = t.x;
  o[1] = t.y;
}
template <int VEC>
__device__ __forceinline__ void ldi(const int* p, int (&o)[VEC]);
template <>
__device__ __forceinline__ void ldi<1>(const int* p, int (&o)[1]) { o[0] = __ldcs(p); }
template <>
__device__ __forceinline__ void ldi<2>(const int* p, int (&o)[2]) {
  const int2 t = __ldcs(reinterpret_cast<const int2*>(p));
  o[0] = t.x;
  o[1] = t.y;
}
template <>
__device__ __forceinline__ void ldi<4>(const int* p, int (&o)[4]) {
  const int4 t = __ldcs(reinterpret_cast<const int4*>(p));
  o[0] = t.x;
  o[1] = t.y;
  o[2] = t.z;
  o[3] = t.w;
}

// Block row a with L lanes, each taking VEC consecutive blocks per step:
// (y0, y1, y2) = sum_s K_as x_adj[s].  Row starts, row lengths and the plane
// stride are multiples of 4 blocks, so every vector load is aligned.
template <typename V, typename A, int VEC, int L>
__device__ __forceinline__ void bsr_row(int a, int sl, const BsrMat<V>& M, const V* x, A& y0, A& y1, A& y2) {
  y0 = y1 = y2 = A(0);
  if (a < M.n_nodes) {
    const int beg = __ldg(M.adj_ptr + a), end = __ldg(M.adj_ptr + a + 1);
    const long long nb = M.nb;
#pragma unroll(VEC == 1 ? 2 : 1)
    for (int s = beg + sl * VEC; s < end; s += L * VEC) {
      int b[VEC];
      ldi<VEC>(M.adj + s, b);
      V k[9][VEC];
#pragma unroll
      for (int p = 0; p < 9; ++p) ldv<V, VEC>(M.val + p * nb + s, k[p]);
#pragma unroll
      for (int t = 0; t < VEC; ++t) {
        const A x0 = (A)x[3 * b[t]], x1 = (A)x[3 * b[t] + 1], x2 = (A)x[3 * b[t] + 2];
        y0 = fma((A)k[0][t], x0, y0);
        y0 = fma((A)k[1][t], x1, y0);
        y0 = fma((A)k[2][t], x2, y0);
        y1 = fma((A)k[3][t], x0, y1);
        y1 = fma((A)k[4][t], x1, y1);
        y1 = fma((A)k[5][t], x2, y1);
        y2 = fma((A)k[6][t], x0, y2);
        y2 = fma((A)k[7][t], x1, y2);
        y2 = fma((A)k[8][t], x2, y2);
      }
    }
  }
  y0 = group_sum<L>(y0);
  y1 = group_sum<L>(y1);
  y2 = group_sum<L>(y2);
}

template <typename V, int VEC, int L>
__global__ void __launch_bounds__(PCG_THREADS) bsr_spmv_kernel(BsrMat<V> M, const V* x, V* y) {
  constexpr int RPW = 32 / L;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
  const int gwarp = tid >> 5, nwarps = nth >> 5;
  const int lane = threadIdx.x & 31, sl = lane % L, grp = lane / L;
  for (int base = gwarp * RPW; base < M.n_nodes; base += nwarps * RPW) {
    const int a = base + grp;
    V y0, y1, y2;
    bsr_row<V, V, VEC, L>(a, sl, M, x, y0, y1, y2);
    if (a < M.n_nodes && sl == 0) {
      y[3 * a] = y0;
      y[3 * a + 1] = y1;
      y[3 * a + 2] = y2;
    }
  }
}

// Block row a of the symmetric form with L lanes:
//   (y0, y1, y2) = sum_{b >= a} K_ab x_b + sum_{b < a} K_ba^T x_b.
// Upper blocks go two at a time (20 floats: five aligned float4 loads, kept in
// L2 for the later rows that read them transposed); a lower block is one
// 40-byte read (five float2) at the position its row b stored it, normally
// still in L2 because row b was streamed a few thousand rows earlier.  The
// first two lower entries of each lane are fetched before the upper loop so
// their index loads overlap it.  Fixed order: bitwise reproducible.
template <int L>
__device__ __forceinline__ void sym_row(int a, int sl, const SymMat& S, const float* x, float& y0, float& y1,
                                        float& y2) {
  y0 = y1 = y2 = 0.f;
  if (a < S.n_nodes) {
    const int l0 = __ldg(S.lptr + a), l1 = __ldg(S.lptr + a + 1);
    int2 pre[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int e = l0 + sl + k * L;
      pre[k] = e < l1 ? __ldcs(S.low + e) : make_int2(-1, 0);
    }
    const int u0 = __ldg(S.uptr + a), u1 = __ldg(S.uptr + a + 1);
    for (int s = u0 + 2 * sl; s < u1; s += 2 * L) {
      const float4* p = reinterpret_cast<const float4*>(S.uval + 10LL * s);
      const float4 q0 = __ldcg(p), q1 = __ldcg(p + 1), q2 = __ldcg(p + 2), q3 = __ldcg(p + 3), q4 = __ldcg(p + 4);
      const int c0 = __float_as_int(q2.y), c1 = __float_as_int(q4.w);
      const float a0 = x[3 * c0], a1 = x[3 * c0 + 1], a2 = x[3 * c0 + 2];
      const float b0 = x[3 * c1], b1 = x[3 * c1 + 1], b2 = x[3 * c1 + 2];
      y0 = fmaf(q0.x, a0, fmaf(q0.y, a1, fmaf(q0.z, a2, y0)));
      y1 = fmaf(q0.w, a0, fmaf(q1.x, a1, fmaf(q1.y, a2, y1)));
      y2 = fmaf(q1.z, a0, fmaf(q1.w, a1, fmaf(q2.x, a2, y2)));
      y0 = fmaf(q2.z, b0, fmaf(q2.w, b1, fmaf(q3.x, b2, y0)));
      y1 = fmaf(q3.y, b0, fmaf(q3.z, b1, fmaf(q3.w, b2, y1)));
      y2 = fmaf(q4.x, b0, fmaf(q4.y, b1, fmaf(q4.z, b2, y2)));
    }
    auto lower = [&](int2 bt) {
      const float2* p = reinterpret_cast<const float2*>(S.uval + 10LL * bt.y);
      const float2 v0 = __ldg(p), v1 = __ldg(p + 1), v2 = __ldg(p + 2), v3 = __ldg(p + 3), v4 = __ldg(p + 4);
      const float b0 = x[3 * bt.x], b1 = x[3 * bt.x + 1], b2 = x[3 * bt.x + 2];
      // K_ba = [v0.x v0.y v1.x; v1.y v2.x v2.y; v3.x v3.y v4.x], y += K_ba^T x_b
      y0 = fmaf(v0.x, b0, fmaf(v1.y, b1, fmaf(v3.x, b2, y0)));
      y1 = fmaf(v0.y, b0, fmaf(v2.x, b1, fmaf(v3.y, b2, y1)));
      y2 = fmaf(v1.x, b0, fmaf(v2.y, b1, fmaf(v4.x, b2, y2)));
    };
#pragma unroll
    for (int k = 0; k < 2; ++k)
      if (pre[k].x >= 0) lower(pre[k]);
    for (int e = l0 + sl + 2 * L; e < l1; e += L) lower(__ldcs(S.low + e));
  }
  y0 = group_sum<L>(y0);
  y1 = group_sum<L>(y1);
  y2 = group_sum<L>(y2);
}

template <int L>
__global__ void __launch_bounds__(PCG_THREADS) sym_spmv_kernel(SymMat S, const float* x, float* y) {
  constexpr int RPW = 32 / L;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
  const int gwarp = tid >> 5, nwarps = nth >> 5;
  const int lane = threadIdx.x & 31, sl = lane % L, grp = lane / L;
  for (int base = gwarp * RPW; base < S.n_nodes; base += nwarps * RPW) {
    const int a = base + grp;
    float y0, y1, y2;
    sym_row<L>(a, sl, S, x, y0, y1, y2);
    if (a < S.n_nodes && sl == 0) {
      y[3 * a] = y0;
      y[3 * a + 1] = y1;
      y[3 * a + 2] = y2;
    }
  }
}

template <typename V>
struct BsrPcgArgs {
  BsrMat<V> M;
  int nd;            // 3 n_nodes
  const V* dinv;     // [nd]
  const V* b;
  V* x;
  V* r;
  V* p;
  V* q;
  double* partials;
  double* totals;
  GridBarrier* bar;
  DevStatus* st;
  PcgOut* out;
  double tol;
  long long max_iter;
  unsigned long long limit_ns;
};

// Jacobi PCG on the node-block form (same recurrence as pcg_kernel).
template <typename V, int L>
__global__ void __launch_bounds__(PCG_THREADS) pcg_bsr_kernel(BsrPcgArgs<V> P) {
  using A = V;
  const int nd = P.nd, n_nodes = P.M.n_nodes;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
  constexpr int RPW = 32 / L;
  const int gwarp = tid >> 5, nwarps = nth >> 5;
  const int lane = threadIdx.x & 31, sl = lane % L, grp = lane / L;
  A rz_p = 0, bb_p = 0;
  for (int i = tid; i < nd; i += nth) {
    const V bi = P.b[i];
    P.x[i] = V(0);
    P.r[i] = bi;
    const V z = bi * P.dinv[i];
    P.p[i] = z;
    rz_p = fma(bi, z, rz_p);
    bb_p = fma(bi, bi, bb_p);
  }
  block_partials<A>(bb_p, rz_p, 2, P.partials, S_RR, S_RZ);
  double red[REDUCE_MAX_NV];
  if (!grid_reduce_sync(P.bar, P.st, P.limit_ns, P.partials, P.totals, S_RR, 2, red)) return;
  A rz = (A)red[1];
  const double bnorm = sqrt(red[0]);
  long long iters = 0;
  double residual = bnorm;
  int status = AXIA_OK;
  if (bnorm >= 1e-30) {
    for (long long it = 0; it < P.max_iter; ++it) {
      iters = it + 1;
      A pq_p = 0;
      for (int base = gwarp * RPW; base < n_nodes; base += nwarps * RPW) {
        const int a = base + grp;
        A y0, y1, y2;
        bsr_row<V, A, 1, L>(a, sl, P.M, P.p, y0, y1, y2);
        if (a < n_nodes && sl == 0) {
          P.q[3 * a] = (V)y0;
          P.q[3 * a + 1] = (V)y1;
          P.q[3 * a + 2] = (V)y2;
          pq_p = fma((A)P.p[3 * a], y0, pq_p);
          pq_p = fma((A)P.p[3 * a + 1], y1, pq_p);
          pq_p = fma((A)P.p[3 * a + 2], y2, pq_p);
        }
      }
      block_partials<A>(pq_p, A(0), 1, P.partials, S_PQ, S_PQ);
      double red[REDUCE_MAX_NV];
      if (!grid_reduce_sync(P.bar, P.st, P.limit_ns, P.partials, P.totals, S_PQ, 1, red)) return;
      const A pq = (A)red[0];
      if (!(fabs((double)pq) >= 1e-30)) {
        status = AXIA_ERR_ZERO_PIVOT;
        break;
      }
      const A alpha = rz / pq;
      A rr_p = 0, rzn_p = 0;
      for (int i = tid; i < nd; i += nth) {
        P.x[i] = fma(alpha, P.p[i], P.x[i]);
        const V ri = fma(-alpha, P.q[i], P.r[i]);
        P.r[i] = ri;
        rr_p = fma(ri, ri, rr_p);
        rzn_p = fma(ri, ri * P.dinv[i], rzn_p);
      }
      block_partials<A>(rr_p, rzn_p, 2, P.partials, S_RR, S_RZ);
      if (!grid_reduce_sync(P.bar, P.st, P.limit_ns, P.partials, P.totals, S_RR, 2, red)) return;
      const A rzn = (A)red[1];
      residual = sqrt(red[0]);
      if (!isfinite(residual)) {
        status = AXIA_ERR_NONFINITE;
        break;
      }
      if (residual <= P.tol * bnorm) break;
      const A beta = rzn / rz;
      rz = rzn;
      for (int i = tid; i < nd; i += nth) P.p[i] = fma(beta, P.p[i], P.r[i] * P.dinv[i]);
      if (!grid_sync(P.bar, P.st, P.limit_ns)) return;
    }
    if (status == AXIA_OK && residual > P.tol * bnorm * 10.0) status = AXIA_ERR_NOT_CONVERGED;
  } else {
    residual = 0.0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    P.out->iters = iters;
    P.out->residual = residual;
    P.out->bnorm = bnorm;
    P.out->status = status;
    P.out->updates = 0;
  }
}

// FP32 CG on the FP32 node-block matrix with FP64 reliable updates (the
// recurrence of pcg_reliable_kernel in pcg.cu on the node-block form): when
// the FP32 residual has dropped by delta since the last update, x += x32 in
// FP64 and r is replaced by the FP64 residual b - K x.
// The rows a system occupies and the blocks that solve it: block rows
// [node0, node1) of the node-block matrix, blocks rank = 0..nblk-1 of a group
// with its own barrier, partial-sum area, totals and result record.
struct SolveRange {
  int node0, node1;
  unsigned rank, nblk;
  double* partials;
  double* totals;
  GridBarrier* bar;
  PcgOut* out;
};

// The coarse solve of the two-level preconditioner, r_c complete:
// y = M r_c, and r_c . y reduced over the group.
__device__ __forceinline__ bool coarse_step(const BsrReliableArgs& P, const CoarseArgs& C, const SolveRange& R,
                                            int gwarp, int nwarps, int lane, float* rz_c) {
  __shared__ __align__(16) float s_rc[COARSE_MAX];
  const float acc = coarse_solve(C, s_rc, gwarp, nwarps, lane);
  block_partials<float>(acc, 0.f, 1, R.partials, S_RC, S_RC, R.nblk, R.rank);
  double red[REDUCE_MAX_NV];
  if (!group_reduce_sync(R.bar, P.st, P.limit_ns, R.partials, R.totals, S_RC, 1, R.nblk, red)) return false;
  *rz_c = (float)red[0];
  return true;
}

template <int L32, int V32, int L64, int V64, bool COARSE = false, bool SYM = false>
__device__ __forceinline__ void reliable_body(const BsrReliableArgs& P, const CoarseArgs& C, const SolveRange& R) {
  const int n0 = R.node0, n1 = R.node1;
  const int i0 = 3 * n0;
  BsrMat<float> M32 = P.M32;
  BsrMat<double> M64 = P.M64;
  M32.n_nodes = n1;  // rows past the range read as empty
  M64.n_nodes = n1;
  const int tid = R.rank * blockDim.x + threadIdx.x, nth = R.nblk * blockDim.x;
  const int gwarp = tid >> 5, nwarps = nth >> 5;
  const int lane = threadIdx.x & 31;
  const int nd = 3 * n1;  // vector loops run over [i0, 3 n1)
  double* const partials = R.partials;
  double* const totals = R.totals;
  float rz_p = 0.f;
  double bb_p = 0.0;
  for (int i = i0 + tid; i < nd; i += nth) {
    const double bi = P.b[i];
    P.x[i] = 0.0;
    const float ri = (float)bi;
    P.r32[i] = ri;
    P.x32[i] = 0.f;
    const float z = ri * P.dinv32[i];
    P.p32[i] = z;
    rz_p = fmaf(ri, z, rz_p);
    bb_p = fma(bi, bi, bb_p);
  }
  block_partials<double>(bb_p, (double)rz_p, 2, partials, S_RR, S_RZ, R.nblk, R.rank);
  double red[REDUCE_MAX_NV];
  if (!group_reduce_sync(R.bar, P.st, P.limit_ns, partials, totals, S_RR, 2, R.nblk, red)) return;
  float rz = (float)red[1];
  const double bnorm = sqrt(red[0]);
  double rmax = bnorm, residual = bnorm;
  long long iters = 0;
  int updates = 0, status = AXIA_OK;
  bool converged = bnorm < 1e-30;
  if (converged) residual = 0.0;
  if constexpr (COARSE) {
    if (!converged) {  // p = D^-1 b + Z M Z^T b
      float rz_c = 0.f;
      coarse_restrict(C, P.r32, gwarp, nwarps, lane);
      if (!group_sync(R.bar, P.st, P.limit_ns, R.nblk)) return;
      if (!coarse_step(P, C, R, gwarp, nwarps, lane, &rz_c)) return;
      rz += rz_c;
      coarse_update_p(C, n0, n1, tid, nth, 0.f, P.r32, P.dinv32, P.p32, true);
      if (!group_sync(R.bar, P.st, P.limit_ns, R.nblk)) return;
    }
  }
  for (long long it = 0; !converged && it < P.max_iter; ++it) {
    iters = it + 1;
    float pq_p = 0.f;
    {
      constexpr int RPW = 32 / L32;
      const int sl = lane % L32, grp = lane / L32;
      for (int base = n0 + gwarp * RPW; base < n1; base += nwarps * RPW) {
        const int a = base + grp;
        float y0, y1, y2;
        if constexpr (SYM) {
          SymMat S = P.S32;
          S.n_nodes = n1;
          sym_row<L32>(a, sl, S, P.p32, y0, y1, y2);
        } else {
          bsr_row<float, float, V32, L32>(a, sl, M32, P.p32, y0, y1, y2);
        }
        if (a < n1 && sl == 0) {
          P.q32[3 * a] = y0;
          P.q32[3 * a + 1] = y1;
          P.q32[3 * a + 2] = y2;
          pq_p = fmaf(P.p32[3 * a], y0, pq_p);
          pq_p = fmaf(P.p32[3 * a + 1], y1, pq_p);
          pq_p = fmaf(P.p32[3 * a + 2], y2, pq_p);
        }
      }
    }
    block_partials<float>(pq_p, 0.f, 1, partials, S_PQ, S_PQ, R.nblk, R.rank);
    double red[REDUCE_MAX_NV];
    if (!group_reduce_sync(R.bar, P.st, P.limit_ns, partials, totals, S_PQ, 1, R.nblk, red)) return;
    const float pq = (float)red[0];
    if (!(fabsf(pq) >= 1e-30f) || !isfinite(pq)) {
      status = isfinite(pq) ? AXIA_ERR_ZERO_PIVOT : AXIA_ERR_NONFINITE;
      break;
    }
    const float alpha = rz / pq;
    float rr_p = 0.f, rzn_p = 0.f;
    if constexpr (COARSE) {
      coarse_update_restrict(C, alpha, P.x32, P.p32, P.q32, P.r32, P.dinv32, gwarp, nwarps, lane, rr_p, rzn_p);
    } else {
      for (int i = i0 + tid; i < nd; i += nth) {
        P.x32[i] = fmaf(alpha, P.p32[i], P.x32[i]);
        const float ri = fmaf(-alpha, P.q32[i], P.r32[i]);
        P.r32[i] = ri;
        rr_p = fmaf(ri, ri, rr_p);
        rzn_p = fmaf(ri, ri * P.dinv32[i], rzn_p);
      }
    }
    block_partials<float>(rr_p, rzn_p, 2, partials, S_RR, S_RZ, R.nblk, R.rank);
    if (!group_reduce_sync(R.bar, P.st, P.limit_ns, partials, totals, S_RR, 2, R.nblk, red)) return;
    float rzn = (float)red[1];
    const double rnorm32 = sqrt(red[0]);
    if (!isfinite(rnorm32)) {
      status = AXIA_ERR_NONFINITE;
      break;
    }
    if (rnorm32 <= P.delta * rmax || rnorm32 <= P.tol * bnorm) {
      for (int i = i0 + tid; i < nd; i += nth) {
        P.x[i] += (double)P.x32[i];
        P.x32[i] = 0.f;
      }
      if (!group_sync(R.bar, P.st, P.limit_ns, R.nblk)) return;
      double rr64_p = 0.0;
      float rz_new_p = 0.f;
      {
        constexpr int RPW = 32 / L64;
        const int sl = lane % L64, grp = lane / L64;
        for (int base = n0 + gwarp * RPW; base < n1; base += nwarps * RPW) {
          const int a = base + grp;
          double y[3];
          bsr_row<double, double, V64, L64>(a, sl, M64, P.x, y[0], y[1], y[2]);
          if (a < n1 && sl == 0) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              const int i = 3 * a + c;
              const double ri = P.b[i] - y[c];
              rr64_p = fma(ri, ri, rr64_p);
              const float r32 = (float)ri;
              P.r32[i] = r32;
              rz_new_p = fmaf(r32, r32 * P.dinv32[i], rz_new_p);
            }
          }
        }
      }
      block_partials<double>(rr64_p, (double)rz_new_p, 2, partials, S_RR, S_RZ, R.nblk, R.rank);
      double red[REDUCE_MAX_NV];
      if (!group_reduce_sync(R.bar, P.st, P.limit_ns, partials, totals, S_RR, 2, R.nblk, red)) return;
      ++updates;
      residual = sqrt(red[0]);
      rzn = (float)red[1];
      rmax = residual;
      if (!isfinite(residual)) {
        status = AXIA_ERR_NONFINITE;
        break;
      }
      if (residual <= P.tol * bnorm) {
        converged = true;
        break;
      }
      if constexpr (COARSE) {  // r was replaced: restrict it again
        coarse_restrict(C, P.r32, gwarp, nwarps, lane);
        if (!group_sync(R.bar, P.st, P.limit_ns, R.nblk)) return;
      }
    }
    if constexpr (COARSE) {
      float rz_c = 0.f;
      if (!coarse_step(P, C, R, gwarp, nwarps, lane, &rz_c)) return;
      rzn += rz_c;
    }
    const float beta = rzn / rz;
    rz = rzn;
    if constexpr (COARSE)
      coarse_update_p(C, n0, n1, tid, nth, beta, P.r32, P.dinv32, P.p32, false);
    else
      for (int i = i0 + tid; i < nd; i += nth) P.p32[i] = fmaf(beta, P.p32[i], P.r32[i] * P.dinv32[i]);
    if (!group_sync(R.bar, P.st, P.limit_ns, R.nblk)) return;
  }
  if (status == AXIA_OK && residual > P.tol * bnorm * 10.0) status = AXIA_ERR_NOT_CONVERGED;
  if (R.rank == 0 && threadIdx.x == 0) {
    R.out->iters = iters;
    R.out->residual = residual;
    R.out->bnorm = bnorm;
    R.out->status = status;
    R.out->updates = updates;
  }
}

// FP64 reliable updates: 4 lanes per block row; 2 blocks per load where the
// register budget allows it (the 4-block FP32 variants run 2 blocks per SM).
constexpr int kL64 = 4;
template <int V32>
__host__ __device__ constexpr int rel_v64() { return V32 >= 4 ? 2 : 1; }

// Blocks per SM: vector loads of 4 blocks need the registers of 2 blocks per SM.
template <int V32>
__host__ __device__ constexpr int rel_min_blocks() { return V32 >= 4 ? 2 : 3; }

template <int L32, int V32, bool COARSE = false, bool SYM = false>
__global__ void __launch_bounds__(PCG_THREADS, rel_min_blocks<V32>()) pcg_bsr_reliable_kernel(BsrReliableArgs P) {
  const SolveRange R{0, P.M64.n_nodes, blockIdx.x, gridDim.x, P.partials, P.totals, P.bar, P.out};
  reliable_body<L32, V32, kL64, rel_v64<V32>(), COARSE, SYM>(P, P.C, R);
}

// Independent systems on disjoint node ranges of one node-block matrix (the
// meshes of axia_gpu_setup_multi): block b belongs to group cta_group[b] and
// solves that group's system with the group's own barrier, partial sums,
// totals and result, so each system converges and exits on its own.
// With the two-level preconditioner every group works on its own mesh's
// restriction chunks and rows of the (block-diagonal) coarse inverse.
template <int L32, int V32, bool COARSE = false>
__global__ void __launch_bounds__(PCG_THREADS, 2)
pcg_group_reliable_kernel(BsrReliableArgs P, const MeshGroup* groups, const int* cta_group, GridBarrier* bars,
                          double* totals4, PcgOut* outs) {
  const int g = cta_group[blockIdx.x];
  const MeshGroup G = groups[g];
  const SolveRange R{G.node0, G.node1, blockIdx.x - (unsigned)G.cta0, (unsigned)G.ncta, P.partials + G.part_off,
                     totals4 + 4 * g, bars + g, outs + g};
  CoarseArgs C = P.C;
  if constexpr (COARSE) {
    C.chunk_lo = G.chunk0;
    C.chunk_hi = G.chunk1;
    C.row0 = G.row0;
    C.row1 = G.row1;
    C.col0 = G.col0;
    C.ldm = G.ldm;
    C.minv += G.moff;
  }
  reliable_body<L32, V32, kL64, 2, COARSE>(P, C, R);
}

// b[d] = f[d] - K_fp u0 for free d, 0 for prescribed d
__global__ void k_build_rhs_full(int64_t nd, const int32_t* ind_of, const double* f, const double* kfu0, double* b) {
  for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < nd; d += (int64_t)gridDim.x * blockDim.x) {
    const int r = ind_of[d];
    b[d] = r >= 0 ? f[d] - kfu0[r] : 0.0;
  }
}
// u = u0 + x on free DOFs (reconstruct, constraint.rs:207-217)
__global__ void k_reconstruct_full(int64_t nd, const int32_t* ind_of, const double* u0, const double* x, double* u) {
  for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < nd; d += (int64_t)gridDim.x * blockDim.x)
    u[d] = ind_of[d] >= 0 ? u0[d] + x[d] : u0[d];
}
// ||b - K x|| partials (FP64), full-DOF form
template <int L>
__global__ void __launch_bounds__(PCG_THREADS) bsr_residual_kernel(BsrMat<double> M, const double* b, const double* x,
                                                                   double* partials) {
  constexpr int RPW = 32 / L;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
  const int gwarp = tid >> 5, nwarps = nth >> 5;
  const int lane = threadIdx.x & 31, sl = lane % L, grp = lane / L;
  double rr = 0.0;
  for (int base = gwarp * RPW; base < M.n_nodes; base += nwarps * RPW) {
    const int a = base + grp;
    double y0, y1, y2;
    bsr_row<double, double, 2, L>(a, sl, M, x, y0, y1, y2);
    if (a < M.n_nodes && sl == 0) {
      const double r0 = b[3 * a] - y0, r1 = b[3 * a + 1] - y1, r2 = b[3 * a + 2] - y2;
      rr = fma(r0, r0, fma(r1, r1, fma(r2, r2, rr)));
    }
  }
  block_partials<double>(rr, 0.0, 1, partials, 0, 0);
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
// Lanes per block row and blocks per lane load.  FP32: 4 blocks per load;
// lanes so that a row of the mesh's mean length takes one or two steps.
// FP64: 2 blocks per load.  Requests outside the instantiated set fall back
// to the automatic choice.
struct RowLayout {
  int lanes, vec;
};
static RowLayout bsr_layout(const axia_ctx* ctx, bool fp32, int lanes_req, int vec_req) {
  const double avg = ctx->n_nodes ? (double)ctx->nbq / (double)ctx->n_nodes : 4.0;  // padded blocks per row
  RowLayout r{0, 0};
  if (fp32 && lanes_req == 0 && vec_req == 0 && ctx->tuned_vec > 0) return RowLayout{ctx->tuned_lanes, ctx->tuned_vec};
  r.vec = (vec_req == 1 || vec_req == 2 || (fp32 && vec_req == 4)) ? vec_req : (fp32 ? 4 : 2);
  const double steps = avg / r.vec;  // vector steps per row
  const int auto_l = steps <= 3 ? 2 : (steps <= 6 ? 4 : (steps <= 12 ? 8 : 16));
  r.lanes = (lanes_req == 2 || lanes_req == 4 || lanes_req == 8 || lanes_req == 16) ? lanes_req : auto_l;
  // instantiated: vec 4 with 2/4/8 lanes, vec 2 with 4/8, vec 1 with 4/8/16
  if (r.vec == 4 && r.lanes == 16) r.lanes = 8;
  if (r.vec == 2 && (r.lanes == 2 || r.lanes == 16)) r.lanes = r.lanes == 2 ? 4 : 8;
  if (r.vec == 1 && r.lanes == 2) r.lanes = 4;
  return r;
}

// Calls f(integral_constant<int, L>, integral_constant<int, VEC>) for an instantiated layout.
template <typename F>
static int with_layout(RowLayout r, F&& f) {
  using std::integral_constant;
  if (r.vec == 4) {
    if (r.lanes == 2) return f(integral_constant<int, 2>{}, integral_constant<int, 4>{});
    if (r.lanes == 4) return f(integral_constant<int, 4>{}, integral_constant<int, 4>{});
    return f(integral_constant<int, 8>{}, integral_constant<int, 4>{});
  }
  if (r.vec == 2) {
    if (r.lanes == 4) return f(integral_constant<int, 4>{}, integral_constant<int, 2>{});
    return f(integral_constant<int, 8>{}, integral_constant<int, 2>{});
  }
  if (r.lanes == 4) return f(integral_constant<int, 4>{}, integral_constant<int, 1>{});
  if (r.lanes == 8) return f(integral_constant<int, 8>{}, integral_constant<int, 1>{});
  return f(integral_constant<int, 16>{}, integral_constant<int, 1>{});
}

// The FP64 subset: 1 or 2 blocks per load (a 4-block FP64 load would be 32 bytes).
template <typename F>
static int with_layout64(RowLayout r, F&& f) {
  using std::integral_constant;
  if (r.vec >= 2) {
    if (r.lanes == 4) return f(integral_constant<int, 4>{}, integral_constant<int, 2>{});
    return f(integral_constant<int, 8>{}, integral_constant<int, 2>{});
  }
  if (r.lanes == 4) return f(integral_constant<int, 4>{}, integral_constant<int, 1>{});
  if (r.lanes == 8) return f(integral_constant<int, 8>{}, integral_constant<int, 1>{});
  return f(integral_constant<int, 16>{}, integral_constant<int, 1>{});
}

static int bsr_lanes(const axia_ctx* ctx, int requested) {
  if (requested == 2 || requested == 4 || requested == 8 || requested == 16) return requested;
  double avg = ctx->n_nodes ? (double)ctx->n_adj / (double)ctx->n_nodes : 1.0;  // blocks per block row
  return avg <= 6 ? 4 : (avg <= 12 ? 8 : 16);
}

template <typename V>
static BsrMat<V> bsr_mat(const axia_ctx* ctx, const V* val) {
  return BsrMat<V>{(int)ctx->n_nodes, ctx->d_qptr, ctx->d_qadj, val, (long long)ctx->nbq};
}

static SymMat sym_mat(const axia_ctx* ctx) {
  return SymMat{(int)ctx->n_nodes, ctx->d_uptr, ctx->d_uval, ctx->d_lptr, ctx->d_low};
}

// Lanes per block row of the symmetric form: about one upper pair or lower
// block per lane and step.
static int sym_lanes(const axia_ctx* ctx, int requested) {
  if (requested == 4 || requested == 8 || requested == 16) return requested;
  const double work = ctx->n_nodes ? (0.5 * (double)ctx->nbu + (double)ctx->nbl) / (double)ctx->n_nodes : 1.0;
  return work <= 12 ? 4 : (work <= 28 ? 8 : 16);
}

static int ensure_full_buffers(axia_ctx* ctx, bool mixed) {
  const size_t nd = (size_t)ctx->ndof;
  if (ctx->full_capacity < nd || (mixed && !ctx->d_xf32)) {
    AXIA_TRY(dev_alloc(ctx, &ctx->d_bf, nd));
    AXIA_TRY(dev_alloc(ctx, &ctx->d_xf, nd));
    AXIA_TRY(dev_alloc(ctx, &ctx->d_rf, nd));
    AXIA_TRY(dev_alloc(ctx, &ctx->d_pf, nd));
    AXIA_TRY(dev_alloc(ctx, &ctx->d_qf, nd));
    if (mixed) {
      AXIA_TRY(dev_alloc(ctx, &ctx->d_xf32, nd));
      AXIA_TRY(dev_alloc(ctx, &ctx->d_rf32, nd));
      AXIA_TRY(dev_alloc(ctx, &ctx->d_pf32, nd));
      AXIA_TRY(dev_alloc(ctx, &ctx->d_qf32, nd));
      AXIA_TRY(dev_alloc(ctx, &ctx->d_zf32, nd));
    }
    ctx->full_capacity = nd;
  }
  return AXIA_OK;
}

template <typename V, int L>
static int launch_bsr_pcg_t(axia_ctx* ctx, BsrPcgArgs<V>& P) {
  auto kern = pcg_bsr_kernel<V, L>;
  int grid = 0;
  AXIA_TRY(coop_grid(ctx, (const void*)kern, P.nd, &grid));
  void* params[] = {&P};
  AXIA_CUDA(ctx, cudaLaunchCooperativeKernel((const void*)kern, dim3(grid), dim3(PCG_THREADS), params, 0, ctx->stream));
  ctx->launches++;
  return AXIA_OK;
}

template <typename V>
static int launch_bsr_pcg(axia_ctx* ctx, BsrPcgArgs<V>& P, int lanes) {
  switch (lanes) {
    case 2: return launch_bsr_pcg_t<V, 2>(ctx, P);
    case 4: return launch_bsr_pcg_t<V, 4>(ctx, P);
    case 16: return launch_bsr_pcg_t<V, 16>(ctx, P);
    default: return launch_bsr_pcg_t<V, 8>(ctx, P);
  }
}

template <int L32, int V32, bool COARSE, bool SYM = false>
static int launch_bsr_rel_t(axia_ctx* ctx, BsrReliableArgs& P) {
  auto kern = pcg_bsr_reliable_kernel<L32, V32, COARSE, SYM>;
  int grid = 0;
  AXIA_TRY(coop_grid(ctx, (const void*)kern, P.nd, &grid));
  void* params[] = {&P};
  AXIA_CUDA(ctx, cudaLaunchCooperativeKernel((const void*)kern, dim3(grid), dim3(PCG_THREADS), params, 0, ctx->stream));
  ctx->launches++;
  return AXIA_OK;
}

// The symmetric form: lanes per block row only (V32 = 4 keeps the register
// budget of two blocks per SM).
static int launch_sym_rel(axia_ctx* ctx, BsrReliableArgs& P, int lanes) {
  const bool c = P.C.n_sub > 0;
  if (lanes == 4) return c ? launch_bsr_rel_t<4, 4, true, true>(ctx, P) : launch_bsr_rel_t<4, 4, false, true>(ctx, P);
  if (lanes == 16) return c ? launch_bsr_rel_t<16, 4, true, true>(ctx, P) : launch_bsr_rel_t<16, 4, false, true>(ctx, P);
  return c ? launch_bsr_rel_t<8, 4, true, true>(ctx, P) : launch_bsr_rel_t<8, 4, false, true>(ctx, P);
}

static int launch_bsr_rel(axia_ctx* ctx, BsrReliableArgs& P, RowLayout r) {
  if (P.C.n_sub > 0)
    return with_layout(
        r, [&](auto l, auto v) { return launch_bsr_rel_t<decltype(l)::value, decltype(v)::value, true>(ctx, P); });
  return with_layout(
      r, [&](auto l, auto v) { return launch_bsr_rel_t<decltype(l)::value, decltype(v)::value, false>(ctx, P); });
}

// Occupancy of the group kernel (blocks per SM) for the grid size of a multi-mesh solve.
int group_kernel_capacity(axia_ctx* ctx, int lanes, int vec, int* per_sm, bool coarse) {
  return with_layout(RowLayout{lanes, vec}, [&](auto l, auto v) {
    const void* kern = coarse ? (const void*)pcg_group_reliable_kernel<decltype(l)::value, decltype(v)::value, true>
                              : (const void*)pcg_group_reliable_kernel<decltype(l)::value, decltype(v)::value, false>;
    AXIA_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, kern, PCG_THREADS, 0));
    return (int)AXIA_OK;
  });
}
// Cooperative launch of the group kernel on ctx->stream (capturable).
int launch_group_reliable(axia_ctx* ctx, BsrReliableArgs& P, const MeshGroup* groups, const int* cta_group,
                          GridBarrier* bars, double* totals4, PcgOut* outs, int grid, int lanes, int vec, bool coarse) {
  void* params[] = {&P, &groups, &cta_group, &bars, &totals4, &outs};
  const void* kern = nullptr;
  with_layout(RowLayout{lanes, vec}, [&](auto l, auto v) {
    kern = coarse ? (const void*)pcg_group_reliable_kernel<decltype(l)::value, decltype(v)::value, true>
                  : (const void*)pcg_group_reliable_kernel<decltype(l)::value, decltype(v)::value, false>;
    return 0;
  });
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(PCG_THREADS);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = ctx->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  AXIA_CUDA(ctx, cudaLaunchKernelExC(&cfg, kern, params));
  ctx->launches++;
  return AXIA_OK;
}

// The layout (lanes, blocks per load) a multi-mesh solve uses for a request.
void group_layout(const axia_ctx* ctx, int lanes_req, int vec_req, int* lanes, int* vec) {
  const RowLayout r = bsr_layout(ctx, true, lanes_req, vec_req);
  *lanes = r.lanes;
  *vec = r.vec;
}

int launch_full_rhs(axia_ctx* ctx, const double* d_f) {
  k_build_rhs_full<<<ctx->sm_count * 8, 256, 0, ctx->stream>>>(ctx->ndof, ctx->d_ind_of, d_f, ctx->d_kfu0, ctx->d_bf);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  return AXIA_OK;
}

int launch_full_reconstruct(axia_ctx* ctx, double* d_u) {
  k_reconstruct_full<<<ctx->sm_count * 8, 256, 0, ctx->stream>>>(ctx->ndof, ctx->d_ind_of, ctx->d_u0, ctx->d_xf, d_u);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  return AXIA_OK;
}

int prepare_full_buffers(axia_ctx* ctx) { return ensure_full_buffers(ctx, true); }

BsrReliableArgs make_reliable_args(axia_ctx* ctx, double rtol, double delta, long long max_iter) {
  return BsrReliableArgs{bsr_mat<float>(ctx, ctx->d_bval32), sym_mat(ctx), bsr_mat<double>(ctx, ctx->d_bval64),
                         (int)ctx->ndof,
                         ctx->d_bdinv32, ctx->d_bf, ctx->d_xf, ctx->d_xf32, ctx->d_rf32, ctx->d_pf32, ctx->d_qf32,
                         ctx->d_zf32, ctx->d_partials, ctx->d_totals, ctx->d_bar, ctx->d_status,
                         (PcgOut*)ctx->d_out, rtol, delta, max_iter, 2000000000ull};
}

static double bsr_residual(axia_ctx* ctx, const double* b, const double* x) {
  const int grid = ctx->sm_count * 4;
  bsr_residual_kernel<4><<<grid, PCG_THREADS, 0, ctx->stream>>>(bsr_mat<double>(ctx, ctx->d_bval64), b, x,
                                                                ctx->d_partials);
  ctx->launches++;
  std::vector<double> h(grid);
  cudaMemcpyAsync(h.data(), ctx->d_partials, grid * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  double s = 0.0;
  for (double v : h) s += v;
  return std::sqrt(s);
}

// Solve on the node-block form: rhs from d_f (full), solution into d_u (full).
int bsr_solve(axia_ctx* ctx, const double* d_f, double* d_u, const axia_solve_opts* opts, axia_solve_info* info) {
  const bool sym = opts->matrix_format == AXIA_FORMAT_BSR3_SYM;
  const bool mixed = opts->precision == AXIA_PREC_MIXED;
  if (sym && (!mixed || !ctx->have_bsr64 || !ctx->have_sym32))
    return set_error(ctx, AXIA_ERR_STATE,
                     "the symmetric node-block solve is mixed precision on AXIA_ASM_BSR64 | AXIA_ASM_SYM32");
  if (!sym && (!ctx->have_bsr64 || (mixed && !ctx->have_bsr32)))
    return set_error(ctx, AXIA_ERR_STATE, "node-block solve needs axia_gpu_assemble_ex with the BSR flags");
  if (opts->preconditioner != AXIA_PRECOND_JACOBI && (opts->preconditioner != AXIA_PRECOND_COARSE || !mixed))
    return set_error(ctx, AXIA_ERR_INVALID_ARG, "the coarse preconditioner needs the mixed node-block solve");
  AXIA_TRY(ensure_full_buffers(ctx, mixed));
  AXIA_TRY(reset_dev_status(ctx));
  const int64_t nd = ctx->ndof;
  k_build_rhs_full<<<ctx->sm_count * 8, 256, 0, ctx->stream>>>(nd, ctx->d_ind_of, d_f, ctx->d_kfu0, ctx->d_bf);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  const long long max_iter = opts->max_iter > 0 ? opts->max_iter : std::max<long long>(4LL * ctx->n_free, 200);
  const unsigned long long limit_ns = 2000000000ull;
  const int lanes = bsr_lanes(ctx, opts->spmv_lanes);
  const RowLayout lay = bsr_layout(ctx, true, opts->spmv_lanes, opts->spmv_vec);
  AXIA_CUDA(ctx, cudaMemsetAsync(ctx->d_bar, 0, sizeof(GridBarrier), ctx->stream));
  PcgOut o{};
  if (!mixed) {
    BsrPcgArgs<double> P{bsr_mat<double>(ctx, ctx->d_bval64), (int)nd, ctx->d_bdinv64, ctx->d_bf, ctx->d_xf,
                         ctx->d_rf, ctx->d_pf, ctx->d_qf, ctx->d_partials, ctx->d_totals, ctx->d_bar,
                         ctx->d_status, (PcgOut*)ctx->d_out, opts->rtol, max_iter, limit_ns};
    AXIA_TRY(timed_launch(ctx, info, [&] { return launch_bsr_pcg<double>(ctx, P, lanes); }));
  } else {
    const double delta = opts->inner_rtol > 0 && opts->inner_rtol < 1 ? opts->inner_rtol : 0.1;
    BsrReliableArgs P{bsr_mat<float>(ctx, ctx->d_bval32), sym_mat(ctx), bsr_mat<double>(ctx, ctx->d_bval64), (int)nd,
                      ctx->d_bdinv32, ctx->d_bf, ctx->d_xf, ctx->d_xf32, ctx->d_rf32, ctx->d_pf32, ctx->d_qf32,
                      ctx->d_zf32, ctx->d_partials, ctx->d_totals, ctx->d_bar, ctx->d_status, (PcgOut*)ctx->d_out, opts->rtol,
                      delta, max_iter, limit_ns};
    if (opts->preconditioner == AXIA_PRECOND_COARSE) {
      AXIA_TRY(coarse_prepare(ctx, opts->coarse_nodes, &P.C));
      AXIA_TRY(reset_dev_status(ctx));
      AXIA_CUDA(ctx, cudaMemsetAsync(ctx->d_bar, 0, sizeof(GridBarrier), ctx->stream));
    }
    if (sym)
      AXIA_TRY(timed_launch(ctx, info, [&] { return launch_sym_rel(ctx, P, sym_lanes(ctx, opts->spmv_lanes)); }));
    else
      AXIA_TRY(timed_launch(ctx, info, [&] { return launch_bsr_rel(ctx, P, lay); }));
  }
  AXIA_TRY(read_out(ctx, &o));
  info->iters = o.iters;
  info->outer_iters = mixed ? o.updates : 1;
  info->residual = o.residual;
  info->bnorm = o.bnorm;
  if (o.status != AXIA_OK) return status_error(ctx, o);
  k_reconstruct_full<<<ctx->sm_count * 8, 256, 0, ctx->stream>>>(nd, ctx->d_ind_of, ctx->d_u0, ctx->d_xf, d_u);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  // the mixed kernels end on an FP64 residual b - K x of the returned x (every
  // convergence test is a reliable update's); the FP64 CG's is a recurrence
  info->true_residual = mixed ? o.residual : bsr_residual(ctx, ctx->d_bf, ctx->d_xf);
  return AXIA_OK;
}

int bsr_spmv_device(axia_ctx* ctx, bool fp32, const void* x, void* y, int lanes_req, int vec_req) {
  if (fp32 ? !ctx->have_bsr32 : !ctx->have_bsr64) return set_error(ctx, AXIA_ERR_STATE, "node-block matrix not assembled");
  const int grid_max = ctx->sm_count * 4;
  if (fp32) {
    const auto M = bsr_mat<float>(ctx, ctx->d_bval32);
    with_layout(bsr_layout(ctx, true, lanes_req, vec_req), [&](auto l, auto v) {
      bsr_spmv_kernel<float, decltype(v)::value, decltype(l)::value>
          <<<grid_max, PCG_THREADS, 0, ctx->stream>>>(M, (const float*)x, (float*)y);
      return 0;
    });
  } else {
    const auto M = bsr_mat<double>(ctx, ctx->d_bval64);
    RowLayout r = bsr_layout(ctx, false, lanes_req, vec_req);
    if (r.vec >= 2 && r.lanes == 2) r.lanes = 4;
    with_layout64(r, [&](auto l, auto v) {
      bsr_spmv_kernel<double, decltype(v)::value, decltype(l)::value>
          <<<grid_max, PCG_THREADS, 0, ctx->stream>>>(M, (const double*)x, (double*)y);
      return 0;
    });
  }
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  return AXIA_OK;
}

int sym_spmv_device(axia_ctx* ctx, const float* x, float* y, int lanes_req) {
  if (!ctx->have_sym32) return set_error(ctx, AXIA_ERR_STATE, "symmetric node-block matrix not assembled");
  const int grid = ctx->sm_count * 4;
  const SymMat S = sym_mat(ctx);
  switch (sym_lanes(ctx, lanes_req)) {
    case 4: sym_spmv_kernel<4><<<grid, PCG_THREADS, 0, ctx->stream>>>(S, x, y); break;
    case 16: sym_spmv_kernel<16><<<grid, PCG_THREADS, 0, ctx->stream>>>(S, x, y); break;
    default: sym_spmv_kernel<8><<<grid, PCG_THREADS, 0, ctx->stream>>>(S, x, y); break;
  }
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  return AXIA_OK;
}

// ---------------------------------------------------------------------------
// Autotuner for the layout of the FP32 inner loop
// ---------------------------------------------------------------------------
// Candidates: the instantiated (lanes, blocks per load) pairs.  Each runs the
// mixed solver's persistent kernel for a fixed number of CG iterations on a
// unit load (ones on free DOFs), timed with CUDA events on the context's
// stream; the fastest per iteration wins.  Results are cached in a text file
// of JSON lines {"key": ..., "lanes": L, "vec": V, "us_per_iter": t}, keyed by
// the device name and the shape of the matrix (nodes per element, reduced
// integration, padded blocks per row, node count bucket).
namespace {

__global__ void k_fill_ones(int64_t n, double* f) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    f[i] = 1.0;
}

std::string tune_key(const axia_ctx* ctx) {
  cudaDeviceProp prop{};
  cudaGetDeviceProperties(&prop, ctx->device);
  const double rb = ctx->n_nodes ? (double)ctx->nbq / (double)ctx->n_nodes : 0.0;
  int bucket = 0;
  for (int64_t n = ctx->n_nodes; n > 1; n >>= 1) ++bucket;
  std::string name(prop.name);
  for (char& c : name)
    if (c == '"' || c == '\\') c = '_';
  return name + "|nn=" + std::to_string(ctx->nn) + "|r=" + std::to_string(ctx->reduced) +
         "|rowblocks=" + std::to_string((int)std::lround(rb)) + "|log2nodes=" + std::to_string(bucket);
}

bool cache_lookup(const char* path, const std::string& key, int* lanes, int* vec) {
  FILE* fh = path ? std::fopen(path, "r") : nullptr;
  if (!fh) return false;
  char line[1024];
  const std::string want = "\"key\": \"" + key + "\"";
  bool found = false;
  while (std::fgets(line, sizeof(line), fh)) {
    const std::string l(line);
    if (l.find(want) == std::string::npos) continue;
    const size_t pl = l.find("\"lanes\": "), pv = l.find("\"vec\": ");
    if (pl == std::string::npos || pv == std::string::npos) continue;
    *lanes = std::atoi(l.c_str() + pl + 9);
    *vec = std::atoi(l.c_str() + pv + 7);
    found = true;  // the last matching line wins
  }
  std::fclose(fh);
  return found;
}

}  // namespace

int bsr_autotune(axia_ctx* ctx, const char* cache_path, int* lanes_out, int* vec_out, double* us_out) {
  if (!ctx->have_bsr32 || !ctx->have_bsr64)
    return set_error(ctx, AXIA_ERR_STATE, "autotune needs axia_gpu_assemble_ex(AXIA_ASM_BSR64 | AXIA_ASM_BSR32)");
  const std::string key = tune_key(ctx);
  int l = 0, v = 0;
  if (cache_lookup(cache_path, key, &l, &v)) {
    const RowLayout r = bsr_layout(ctx, true, l, v);
    if (r.lanes == l && r.vec == v) {
      ctx->tuned_lanes = l;
      ctx->tuned_vec = v;
      *lanes_out = l;
      *vec_out = v;
      if (us_out) *us_out = 0.0;
      return AXIA_OK;
    }
  }
  AXIA_TRY(ensure_full_buffers(ctx, true));
  double* d_ones = nullptr;
  AXIA_TRY(dev_alloc(ctx, &d_ones, (size_t)ctx->ndof));
  k_fill_ones<<<ctx->sm_count * 4, 256, 0, ctx->stream>>>(ctx->ndof, d_ones);
  int st = launch_full_rhs(ctx, d_ones);
  const RowLayout cands[] = {{8, 4}, {4, 4}, {2, 4}, {8, 2}, {4, 2}, {16, 1}, {8, 1}, {4, 1}};
  const long long iters = 40;
  double best = 1e300;
  RowLayout pick{0, 0};
  cudaEvent_t a = nullptr, b = nullptr;
  if (st == AXIA_OK && (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess))
    st = set_error(ctx, AXIA_ERR_CUDA, "autotune events");
  for (const RowLayout& c : cands) {
    if (st != AXIA_OK) break;
    BsrReliableArgs P = make_reliable_args(ctx, 1e-30, 0.01, iters);
    float best_c = 1e30f;
    for (int rep = 0; rep < 2 && st == AXIA_OK; ++rep) {
      if ((st = reset_dev_status(ctx)) != AXIA_OK) break;
      cudaMemsetAsync(ctx->d_bar, 0, sizeof(GridBarrier), ctx->stream);
      cudaEventRecord(a, ctx->stream);
      st = launch_bsr_rel(ctx, P, c);
      cudaEventRecord(b, ctx->stream);
      if (st != AXIA_OK) break;
      PcgOut o{};
      if ((st = read_out(ctx, &o)) != AXIA_OK) break;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, a, b);
      best_c = std::min(best_c, ms / (float)std::max<long long>(o.iters, 1));
    }
    if (st == AXIA_OK && best_c < best) {
      best = best_c;
      pick = c;
    }
  }
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  dev_free(d_ones);
  if (st != AXIA_OK) return st;
  ctx->tuned_lanes = pick.lanes;
  ctx->tuned_vec = pick.vec;
  *lanes_out = pick.lanes;
  *vec_out = pick.vec;
  if (us_out) *us_out = best * 1e3;
  if (cache_path) {
    if (FILE* fh = std::fopen(cache_path, "a")) {
      std::fprintf(fh, "{\"key\": \"%s\", \"lanes\": %d, \"vec\": %d, \"us_per_iter\": %.3f}\n", key.c_str(),
                   pick.lanes, pick.vec, best * 1e3);
      std::fclose(fh);
    }
  }
  return AXIA_OK;
}
