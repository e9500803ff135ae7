// element.cuh -- C3D8 / C3D20(R) / C3D4 / C3D10 element stiffness on the
// device, one warp per element.
//
// Restates, with an isotropic closed form for the contraction, the
// reference's hex8_stiffness (solver/src/elem.rs:194-219), hex20_stiffness
// (solver/src/quadratic.rs:122-146), tet4_stiffness (elem.rs:221-248, one
// point, weight 1/6) and tet10_stiffness (quadratic.rs:607-627, 4 points,
// weights 1/24): Ke = sum_gp w det(J) B^T D B.
//
// For isotropic D (d_iso_3d, elem.rs:41-59) the 3x3 block of nodes (a, b) is
//   K_ab[i][j] = lam A_ab[i][j] + mu A_ab[j][i] + mu delta_ij tr(A_ab),
//   A_ab[i][j] = sum_gp (w / det J) c_a[i] c_b[j],   c_a = adj(J)^T-part of dN_a,
// where dN_a/dx = c_a / det J (J^-1 = adj(J) / det J, invert3 elem.rs:10-29).
// Only the blocks a <= b are integrated (Ke is symmetric); lanes own fixed
// entries of that upper triangle so all 32 lanes stay busy on the FP64 pipe.
//
// Shared-memory layout per warp (doubles):
//   X[3NN] nodal coordinates, J[NG*9], G[NG*9] (cofactor matrix), S[NG] w/det,
//   U = union{ C[NG*3NN] + H[NG*3NN] ; KE[(3NN)^2] }, A[NE], TR[NB]
// The finished Ke (row-major, node-major DOF order as element_ke returns it,
// elem.rs:337-342) leaves shared memory through a TMA bulk store.
#pragma once

#include "common.cuh"

template <int NN, int NG>
struct ElemTraits {
  static constexpr int NDOF = 3 * NN;
  static constexpr int NB = NN * (NN + 1) / 2;          // node pairs a <= b
  static constexpr int NE = 9 * NN * (NN - 1) / 2 + 6 * NN;  // unique entries
  static constexpr int KE = NDOF * NDOF;
  static constexpr int CH = (NE + 31) / 32 > 32 ? 30 : (NE + 31) / 32;  // accumulators per lane
  static constexpr int NCHUNK = (NE + 32 * CH - 1) / (32 * CH);
  static constexpr int U = (2 * NG * NDOF > KE) ? 2 * NG * NDOF : KE;
  // per-warp doubles, every section a multiple of 2 doubles (16 B alignment)
  static constexpr __host__ __device__ int R2(int v) { return (v + 1) & ~1; }
  static constexpr int OFF_X = 0;
  static constexpr int OFF_J = OFF_X + R2(NDOF);
  static constexpr int OFF_G = OFF_J + R2(NG * 9);
  static constexpr int OFF_S = OFF_G + R2(NG * 9);
  static constexpr int OFF_U = OFF_S + R2(NG);
  static constexpr int OFF_A = OFF_U + R2(U);
  static constexpr int OFF_TR = OFF_A + R2(NE);
  static constexpr int WARP_DOUBLES = OFF_TR + R2(NB);
};

// Per-entry table: e0 = hidx | cidx << 8 | (i==j) << 16, e1 = kT | blk << 16.
// Per-block table: base entry | diag flag << 16 (trace = A[base]+A[base+d1]+A[base+d2]).
struct ElemTables {
  const double* dn;      // [NG][NN][3] dN/dxi at the Gauss points
  const double* w;       // [NG]
  const int* e0;         // [NE]
  const int* e1;         // [NE]
  const int* blk;        // [NB]
};

struct ElemArgs {
  int64_t n_elem;
  const int32_t* conn;   // [n_elem][NN] (global node ids) -- or null when xyz given
  const double* coords;  // [n_nodes][3]
  const double* xyz;     // [n_elem][NN][3] when conn == null (batched element_ke)
  const double* e_elem;  // [n_elem] or null
  double e_const;
  double c_lam, c_mu;    // lam = E c_lam, mu = E c_mu
  double* ke_out;        // [n_elem][KE]
  double* vol_out;       // [n_elem] or null
  DevStatus* status;
  int ke_dw;             // double-word kernel only: Ke entries as FP32 pairs (h, l) instead of FP64
};

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

// Every lane that wrote the source calls fence_async_smem() before the warp
// syncs and one lane issues the store.
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void bulk_store_s2g(double* gdst, const double* ssrc, unsigned bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst),
               "r"(smem_u32(ssrc)), "r"(bytes)
               : "memory");
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_all() {
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

template <int NN, int NG, int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
element_ke_kernel(ElemArgs args, ElemTables tab) {
  using T = ElemTraits<NN, NG>;
  extern __shared__ __align__(16) double smem[];
  double* s_dn = smem;                       // [NG*NN*3]
  double* s_w = s_dn + NG * NN * 3;          // [NG]
  const int tab_doubles = T::R2(NG * NN * 3 + NG);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* W = smem + tab_doubles + warp * T::WARP_DOUBLES;
  double* X = W + T::OFF_X;
  double* J = W + T::OFF_J;
  double* G = W + T::OFF_G;
  double* S = W + T::OFF_S;
  double* C = W + T::OFF_U;
  double* H = C + NG * T::NDOF;
  double* KEs = W + T::OFF_U;
  double* A = W + T::OFF_A;
  double* TR = W + T::OFF_TR;

  for (int t = threadIdx.x; t < NG * NN * 3; t += blockDim.x) s_dn[t] = tab.dn[t];
  for (int t = threadIdx.x; t < NG; t += blockDim.x) s_w[t] = tab.w[t];
  __syncthreads();

  // lane-owned entries of the upper triangle
  int my_e0[T::NCHUNK * T::CH];
#pragma unroll
  for (int m = 0; m < T::NCHUNK * T::CH; ++m) {
    int k = lane + 32 * m;
    my_e0[m] = k < T::NE ? tab.e0[k] : -1;
  }

  const int64_t warps_total = (int64_t)gridDim.x * WARPS;
  for (int64_t e = (int64_t)blockIdx.x * WARPS + warp; e < args.n_elem; e += warps_total) {
    // 1. nodal coordinates
    for (int t = lane; t < T::NDOF; t += 32) {
      double v;
      if (args.conn) {
        int node = __ldg(args.conn + e * NN + t / 3);
        v = __ldg(args.coords + 3 * (int64_t)node + (t % 3));
      } else {
        v = __ldg(args.xyz + e * T::NDOF + t);
      }
      if (!isfinite(v)) record_error(args.status, e, AXIA_ERR_NONFINITE);
      X[t] = v;
    }
    const double E = args.e_elem ? __ldg(args.e_elem + e) : args.e_const;
    __syncwarp();
    // 2. J[g][q][p] = sum_a dN_a/dxi_p x_a,q (elem.rs:175-181)
    for (int t = lane; t < NG * 9; t += 32) {
      int g = t / 9, q = (t % 9) / 3, p = t % 3;
      const double* dn = s_dn + g * NN * 3;
      double s = 0.0;
#pragma unroll 4
      for (int a = 0; a < NN; ++a) s = fma(dn[3 * a + p], X[3 * a + q], s);
      J[t] = s;
    }
    __syncwarp();
    // 3. cofactor matrix b[i][j] (invert3 before the 1/det scaling, elem.rs:18-26)
    for (int t = lane; t < NG * 9; t += 32) {
      int g = t / 9, i = (t % 9) / 3, j = t % 3;
      const double* a = J + 9 * g;
      int j1 = (j + 1) % 3, j2 = (j + 2) % 3, i1 = (i + 1) % 3, i2 = (i + 2) % 3;
      G[t] = a[3 * j1 + i1] * a[3 * j2 + i2] - a[3 * j1 + i2] * a[3 * j2 + i1];
    }
    __syncwarp();
    double vol_part = 0.0;
    for (int g = lane; g < NG; g += 32) {
      const double* a = J + 9 * g;
      const double* b = G + 9 * g;
      double det = a[0] * b[0] + a[1] * b[3] + a[2] * b[6];
      if (!(fabs(det) >= 1e-18)) {
        record_error(args.status, e, isfinite(det) ? AXIA_ERR_SINGULAR_JACOBIAN : AXIA_ERR_NONFINITE);
        det = 1.0;
      } else if (det <= 0.0) {
        record_error(args.status, e, AXIA_ERR_NEG_JACOBIAN);
      }
      S[g] = s_w[g] / det;
      vol_part += s_w[g] * det;
    }
    if (!(E > 0.0)) {
      if (lane == 0) record_error(args.status, e, AXIA_ERR_MATERIAL);
    }
    if (args.vol_out) {
      vol_part = warp_sum(vol_part);
      if (lane == 0) args.vol_out[e] = vol_part;
    }
    // the previous element's bulk store still reads the C/H/KE union
    if (lane == 0) bulk_wait_read();
    __syncwarp();
    // 4. c_a[i] = sum_p b[p][i] dN_a/dxi_p, h = (w/det) c
    for (int t = lane; t < NG * T::NDOF; t += 32) {
      int g = t / T::NDOF, r = t % T::NDOF, a = r / 3, i = r % 3;
      const double* b = G + 9 * g;
      const double* dn = s_dn + (g * NN + a) * 3;
      double c = fma(b[i], dn[0], fma(b[3 + i], dn[1], b[6 + i] * dn[2]));
      C[t] = c;
      H[t] = S[g] * c;
    }
    __syncwarp();
    // 5. A_ab[i][j] = sum_g h_a[i] c_b[j] for the lane's entries
#pragma unroll
    for (int ch = 0; ch < T::NCHUNK; ++ch) {
      double acc[T::CH];
#pragma unroll
      for (int m = 0; m < T::CH; ++m) acc[m] = 0.0;
      for (int g = 0; g < NG; ++g) {
        const double* Hg = H + g * T::NDOF;
        const double* Cg = C + g * T::NDOF;
#pragma unroll
        for (int m = 0; m < T::CH; ++m) {
          int code = my_e0[ch * T::CH + m];
          if (code >= 0) acc[m] = fma(Hg[code & 0xff], Cg[(code >> 8) & 0xff], acc[m]);
        }
      }
#pragma unroll
      for (int m = 0; m < T::CH; ++m) {
        int k = lane + 32 * (ch * T::CH + m);
        if (k < T::NE) A[k] = acc[m];
      }
    }
    __syncwarp();
    // 6. block traces
    for (int b = lane; b < T::NB; b += 32) {
      int v = __ldg(tab.blk + b);
      int base = v & 0xffff;
      bool dg = (v >> 16) & 1;
      TR[b] = dg ? A[base] + A[base + 3] + A[base + 5] : A[base] + A[base + 4] + A[base + 8];
    }
    __syncwarp();
    // 7. K_ab[i][j] = lam A[i][j] + mu A[j][i] + mu delta_ij tr, both triangles
    const double lam = E * args.c_lam, mu = E * args.c_mu;
    for (int k = lane; k < T::NE; k += 32) {
      int c0 = __ldg(tab.e0 + k), c1 = __ldg(tab.e1 + k);
      int hi = c0 & 0xff, ci = (c0 >> 8) & 0xff;
      double v = fma(lam, A[k], mu * A[c1 & 0xffff]);
      if ((c0 >> 16) & 1) v = fma(mu, TR[c1 >> 16], v);
      KEs[hi * T::NDOF + ci] = v;
      KEs[ci * T::NDOF + hi] = v;
    }
    fence_async_smem();
    __syncwarp();
    // 8. bulk store of the finished Ke; a bulk copy needs 16-byte aligned ends, which
    // an odd Ke size (C3D15: 45 x 45 doubles) does not give every element, so that
    // one is stored by the warp
    if constexpr (T::KE % 2 == 0) {
      if (lane == 0) bulk_store_s2g(args.ke_out + e * T::KE, KEs, (unsigned)(T::KE * sizeof(double)));
    } else {
      for (int k = lane; k < T::KE; k += 32) args.ke_out[e * T::KE + k] = KEs[k];
    }
    __syncwarp();
  }
  if (lane == 0) bulk_wait_all();
  __syncwarp();
}

template <int NN, int NG>
constexpr size_t element_smem_bytes(int warps) {
  return (size_t)(ElemTraits<NN, NG>::R2(NG * NN * 3 + NG) + warps * ElemTraits<NN, NG>::WARP_DOUBLES) *
         sizeof(double);
}
