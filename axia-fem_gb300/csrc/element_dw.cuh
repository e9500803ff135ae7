// element_dw.cuh -- C3D8, C3D20 and C3D20R element stiffness with the Gauss
// loop on the FP32 pipe in double-word arithmetic (dword.cuh), one warp per
// element: element_ke_dw_kernel (C3D8, lanes own Ke entries) and
// element_ke_dw_pair_kernel (20 nodes, lanes own 3x3 node blocks).
//
// The same restatement as element_ke_kernel (element.cuh; the reference's
// hex8_stiffness, solver/src/elem.rs:194-219): Ke = sum_gp w det(J) B^T D B
// in the isotropic closed form K_ab = lam A_ab + mu A_ab^T + mu tr(A_ab) I,
// A_ab = sum_gp (w / det J) c_a c_b^T, with the same tables, lane-owned
// upper-triangle entries and shared-memory layout.  What differs:
//   * the coordinates enter as differences from the element's first node
//     (exact in FP64 for the nodes of one element), scaled by 2^-k so the
//     largest is in [1/2, 1): every intermediate is then of order one, far
//     inside the FP32 exponent range, and the element's distance from the
//     origin costs no accuracy.  Ke scales by 2^k (folded into lam and mu)
//     and det J by 2^3k, both exactly;
//   * J = dN^T X, the cofactors, det J, w / det J, c, h, A, the traces and
//     the Ke entries in double words (compensated dot products);
//   * det J for the Jacobian checks and the volume in FP64 (one add from the
//     double word), so the singular / negative tests keep their meaning;
//   * Ke leaves as double words for the assembly's gather, which sums them in
//     double words too (ElemArgs::ke_dw), or as FP64 for callers of the
//     element stiffness (one FP64 add of two exactly re-encoded FP32 parts
//     per unique entry).
// About 6 FP64 warp instructions per element remain, against about 150 in
// element_ke_kernel (4,900 FP64 operations), which GB300's FP64 pipe (about
// 1/75 of the FP32 rate) bounds.  This kernel is bound by instruction issue
// instead (about 3,700 warp instructions per element, 12 FP32 operations per
// double-word multiply-add).  Accuracy: within about 3e-14 of max|Ke| of the
// exact element stiffness for well-shaped to moderately distorted elements
// (the FP64 kernel: about 1e-15).
#pragma once

#include "dword.cuh"
#include "element.cuh"

template <int NN, int NG>
struct ElemDwTraits {
  using T = ElemTraits<NN, NG>;
  // dN/dxi, the weights and the material factors lam / E, mu / E as double words
  static constexpr int TAB = T::R2(NG * NN * 3 + NG + 2);
};

template <int NN, int NG>
constexpr size_t element_dw_smem_bytes(int warps) {
  return (size_t)(ElemDwTraits<NN, NG>::TAB + warps * ElemTraits<NN, NG>::WARP_DOUBLES) * sizeof(double);
}

// Three blocks of 8 warps per SM (their shared memory fits three).
template <int NN, int NG, int WARPS>
__global__ void __launch_bounds__(WARPS * 32, 3)
element_ke_dw_kernel(ElemArgs args, ElemTables tab) {
  using T = ElemTraits<NN, NG>;
  using D = ElemDwTraits<NN, NG>;
  extern __shared__ __align__(16) double smem[];
  dw* s_dnw = reinterpret_cast<dw*>(smem);                    // [NG*NN*3]
  dw* s_w = s_dnw + NG * NN * 3;                              // [NG]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* W = smem + D::TAB + warp * T::WARP_DOUBLES;
  dw* Xw = reinterpret_cast<dw*>(W + T::OFF_X);
  dw* J = reinterpret_cast<dw*>(W + T::OFF_J);
  dw* G = reinterpret_cast<dw*>(W + T::OFF_G);
  dw* S = reinterpret_cast<dw*>(W + T::OFF_S);
  dw* C = reinterpret_cast<dw*>(W + T::OFF_U);
  dw* H = C + NG * T::NDOF;
  double* KEs = W + T::OFF_U;
  dw* A = reinterpret_cast<dw*>(W + T::OFF_A);
  dw* TR = reinterpret_cast<dw*>(W + T::OFF_TR);

  for (int t = threadIdx.x; t < NG * NN * 3; t += blockDim.x) {
    s_dnw[t] = dw_from_double(tab.dn[t]);
  }
  for (int t = threadIdx.x; t < NG; t += blockDim.x) s_w[t] = dw_from_double(tab.w[t]);
  dw* s_cm = s_w + NG;  // [2]: c_lam, c_mu
  if (threadIdx.x == 0) {
    s_cm[0] = dw_from_double(args.c_lam);
    s_cm[1] = dw_from_double(args.c_mu);
  }
  __syncthreads();

  // lane-owned entries k = lane + 32 m: byte offsets of h_a[i] and c_b[j] in
  // the first Gauss point's rows, so the accumulation loop does no decoding or
  // predication (entries past NE use entry 0's and are not stored)
  constexpr int NM = T::NCHUNK * T::CH;
  static_assert(NM <= 16, "per-lane offsets are meant for the C3D8 entry count");
  const char* const base = reinterpret_cast<const char*>(smem);
  int hoff[NM], coff[NM];
#pragma unroll
  for (int m = 0; m < NM; ++m) {
    const int k = lane + 32 * m;
    const int code = __ldg(tab.e0 + (k < T::NE ? k : 0));
    hoff[m] = (int)(reinterpret_cast<const char*>(H + (code & 0xff)) - base);
    coff[m] = (int)(reinterpret_cast<const char*>(C + ((code >> 8) & 0xff)) - base);
  }

  const int64_t warps_total = (int64_t)gridDim.x * WARPS;
  for (int64_t e = (int64_t)blockIdx.x * WARPS + warp; e < args.n_elem; e += warps_total) {
    // 1. coordinates relative to node 0; 2^k above the largest difference
    constexpr int PER = (T::NDOF + 31) / 32;
    double dif[PER];
    int emax = 0;
#pragma unroll
    for (int s = 0; s < PER; ++s) {
      const int t = lane + 32 * s;
      dif[s] = 0.0;
      if (t < T::NDOF) {
        double v, r;
        if (args.conn) {
          const int node = __ldg(args.conn + e * NN + t / 3);
          const int node0 = __ldg(args.conn + e * NN);
          v = __ldg(args.coords + 3 * (int64_t)node + (t % 3));
          r = __ldg(args.coords + 3 * (int64_t)node0 + (t % 3));
        } else {
          v = __ldg(args.xyz + e * T::NDOF + t);
          r = __ldg(args.xyz + e * T::NDOF + (t % 3));
        }
        if (!finite_bits(v)) record_error(args.status, e, AXIA_ERR_NONFINITE);
        dif[s] = v - r;
        const int be = (int)((__double_as_longlong(dif[s]) >> 52) & 0x7ff);
        emax = max(emax, be == 0x7ff ? 0 : be);
      }
    }
    emax = __reduce_max_sync(0xffffffffu, emax);
    // |dif| < 2^(emax - 1022); an all-zero or non-finite element keeps k = 0
    const int k = emax == 0 ? 0 : min(max(emax - 1022, -1000), 1000);
    const double E = args.e_elem ? __ldg(args.e_elem + e) : args.e_const;
#pragma unroll
    for (int s = 0; s < PER; ++s) {
      const int t = lane + 32 * s;
      if (t < T::NDOF) Xw[t] = dw_split_scaled(dif[s], k);
    }
    __syncwarp();
    // 2. J[g][q][p] = sum_a dN_a/dxi_p x_a,q (elem.rs:175-181)
    for (int t = lane; t < NG * 9; t += 32) {
      const int g = t / 9, q = (t % 9) / 3, p = t % 3;
      const dw* dn = s_dnw + g * NN * 3;
      dw_acc s;
#pragma unroll
      for (int a = 0; a < NN; ++a) dw_fma(s, dn[3 * a + p], Xw[3 * a + q]);
      J[t] = dw_value(s);
    }
    __syncwarp();
    // 3. cofactor matrix b[i][j] (invert3 before the 1/det scaling, elem.rs:18-26)
    for (int t = lane; t < NG * 9; t += 32) {
      const int g = t / 9, i = (t % 9) / 3, j = t % 3;
      const dw* a = J + 9 * g;
      const int j1 = (j + 1) % 3, j2 = (j + 2) % 3, i1 = (i + 1) % 3, i2 = (i + 2) % 3;
      dw_acc s;
      dw_fma(s, a[3 * j1 + i1], a[3 * j2 + i2]);
      dw_fma(s, dw_neg(a[3 * j1 + i2]), a[3 * j2 + i1]);
      G[t] = dw_value(s);
    }
    __syncwarp();
    double vol_part = 0.0;
    for (int g = lane; g < NG; g += 32) {
      const dw* a = J + 9 * g;
      const dw* b = G + 9 * g;
      dw_acc s;
      dw_fma(s, a[0], b[0]);
      dw_fma(s, a[1], b[3]);
      dw_fma(s, a[2], b[6]);
      const dw det_s = dw_value(s);                       // det of the scaled element
      double det = dw_to_double(det_s);
      if (k >= -340 && k <= 340) {
        det *= pow2(3 * k);
      } else {
        const double p2k = pow2(k);
        det = det * p2k * p2k * p2k;
      }
      const double w = tab.w[g];
      if (!(fabs(det) >= 1e-18)) {
        record_error(args.status, e, isfinite(det) ? AXIA_ERR_SINGULAR_JACOBIAN : AXIA_ERR_NONFINITE);
        S[g] = s_w[g];
      } else {
        if (det <= 0.0) record_error(args.status, e, AXIA_ERR_NEG_JACOBIAN);
        S[g] = dw_div(s_w[g], det_s);
      }
      vol_part += w * det;
    }
    if (!(__double_as_longlong(E) > 0 && __double_as_longlong(E) <= 0x7ff0000000000000ll)) {  // !(E > 0)
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
      const int g = t / T::NDOF, r = t % T::NDOF, a = r / 3, i = r % 3;
      const dw* b = G + 9 * g;
      const dw* dn = s_dnw + (g * NN + a) * 3;
      dw_acc s;
      dw_fma(s, b[i], dn[0]);
      dw_fma(s, b[3 + i], dn[1]);
      dw_fma(s, b[6 + i], dn[2]);
      const dw c = dw_value(s);
      C[t] = c;
      H[t] = dw_mul(S[g], c);
    }
    __syncwarp();
    // 5. A_ab[i][j] = sum_g h_a[i] c_b[j] for the lane's entries
#pragma unroll
    for (int ch = 0; ch < T::NCHUNK; ++ch) {
      dw_acc acc[T::CH];
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        const int step = g * T::NDOF * (int)sizeof(dw);
#pragma unroll
        for (int m = 0; m < T::CH; ++m)
          dw_fma(acc[m], *reinterpret_cast<const dw*>(base + hoff[ch * T::CH + m] + step),
                 *reinterpret_cast<const dw*>(base + coff[ch * T::CH + m] + step));
      }
#pragma unroll
      for (int m = 0; m < T::CH; ++m) {
        const int kk = lane + 32 * (ch * T::CH + m);
        if (kk < T::NE) A[kk] = dw_value(acc[m]);
      }
    }
    __syncwarp();
    // 6. block traces
    for (int b = lane; b < T::NB; b += 32) {
      const int v = __ldg(tab.blk + b);
      const int base = v & 0xffff;
      const bool dg = (v >> 16) & 1;
      dw_acc s;
      dw_add(s, A[base]);
      dw_add(s, A[base + (dg ? 3 : 4)]);
      dw_add(s, A[base + (dg ? 5 : 8)]);
      TR[b] = dw_value(s);
    }
    __syncwarp();
    // 7. K_ab[i][j] = lam A[i][j] + mu A[j][i] + mu delta_ij tr, both triangles;
    // lam and mu carry the 2^k of the scaled coordinates
    dw lam, mu;
    if (k >= -100 && k <= 100) {
      const dw Ew = dw_split_scaled(E, 0);
      lam = dw_scale(dw_mul(Ew, s_cm[0]), k);
      mu = dw_scale(dw_mul(Ew, s_cm[1]), k);
    } else {
      lam = dw_from_double(E * args.c_lam * pow2(k));
      mu = dw_from_double(E * args.c_mu * pow2(k));
    }
    for (int kk = lane; kk < T::NE; kk += 32) {
      const int c0 = __ldg(tab.e0 + kk), c1 = __ldg(tab.e1 + kk);
      const int hi = c0 & 0xff, ci = (c0 >> 8) & 0xff;
      dw_acc s;
      dw_fma(s, lam, A[kk]);
      dw_fma(s, mu, A[c1 & 0xffff]);
      if ((c0 >> 16) & 1) dw_fma(s, mu, TR[c1 >> 16]);
      const dw v = dw_value(s);
      if (args.ke_dw) {
        dw* KEw = reinterpret_cast<dw*>(KEs);
        KEw[hi * T::NDOF + ci] = v;
        KEw[ci * T::NDOF + hi] = v;
      } else {
        const double vd = dw_to_double(v);
        KEs[hi * T::NDOF + ci] = vd;
        KEs[ci * T::NDOF + hi] = vd;
      }
    }
    fence_async_smem();
    __syncwarp();
    // 8. bulk store of the finished Ke (KE is even for these kinds: 16-byte ends)
    static_assert(T::KE % 2 == 0, "bulk store needs an even Ke size");
    if (lane == 0) bulk_store_s2g(args.ke_out + e * T::KE, KEs, (unsigned)(T::KE * sizeof(double)));
    __syncwarp();
  }
  if (lane == 0) bulk_wait_all();
  __syncwarp();
}

// C3D20 / C3D20R in double words, one warp per element, each lane owning
// whole 3x3 node blocks: A_ab = sum_g h_a c_b^T for node pairs a <= b (210
// for 20 nodes, 7 rounds of 32 lanes), from which the lane forms K_ab =
// lam A_ab + mu A_ab^T + mu tr(A_ab) I in registers and stores K_ab and its
// mirror K_ba straight to global memory.  Against the per-entry ownership of
// element_ke_dw_kernel (which at 1,830 entries and 27 Gauss points had shared
// memory for 4 warps per SM and measured slower than the FP64 loop) this
// needs no A, trace or entry tables in shared memory, and each Gauss point
// costs a lane 7 shared loads (c_a, c_b, w/det) for 9 multiply-adds instead
// of 2 per multiply-add.  h_a = (w/det) c_a is formed by the lane (3
// double-word products per Gauss point, the same values a stored h would
// hold), so only c is kept per Gauss point: 15.6 KB per warp, 14 warps per
// SM.  The Jacobians share c's space (they are dead before c is formed).  On
// a diagonal pair (a == b) the entries i <= j are formed and mirrored, so Ke
// is exactly symmetric like the other kernels' output.
template <int NN, int NG>
struct ElemDwPairTraits {
  using T = ElemTraits<NN, NG>;
  static constexpr int NR = (T::NB + 31) / 32;  // rounds of node pairs per lane
  static constexpr int TAB = T::R2(NG * NN * 3 + NG + 2);
  static constexpr int OFF_X = 0;
  static constexpr int OFF_G = OFF_X + T::R2(T::NDOF);
  static constexpr int OFF_S = OFF_G + T::R2(NG * 9);
  static constexpr int OFF_C = OFF_S + T::R2(NG);
  static constexpr int WARP_UNITS = OFF_C + T::R2(NG * T::NDOF);  // 8-byte units per warp
  static_assert(NG * 9 <= NG * T::NDOF, "the Jacobians fit in c's space");
};

template <int NN, int NG>
constexpr size_t element_dw_pair_smem_bytes(int warps) {
  using D = ElemDwPairTraits<NN, NG>;
  return (size_t)(D::TAB + warps * D::WARP_UNITS) * sizeof(double);
}

template <int NN, int NG, int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
element_ke_dw_pair_kernel(ElemArgs args, ElemTables tab) {
  using T = ElemTraits<NN, NG>;
  using D = ElemDwPairTraits<NN, NG>;
  extern __shared__ __align__(16) double smem[];
  dw* s_dnw = reinterpret_cast<dw*>(smem);  // [NG*NN*3]
  dw* s_w = s_dnw + NG * NN * 3;            // [NG]
  dw* s_cm = s_w + NG;                      // [2]: c_lam, c_mu
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* W = smem + D::TAB + warp * D::WARP_UNITS;
  dw* Xw = reinterpret_cast<dw*>(W + D::OFF_X);
  dw* G = reinterpret_cast<dw*>(W + D::OFF_G);
  dw* S = reinterpret_cast<dw*>(W + D::OFF_S);
  dw* C = reinterpret_cast<dw*>(W + D::OFF_C);
  dw* J = C;
  for (int t = threadIdx.x; t < NG * NN * 3; t += blockDim.x) s_dnw[t] = dw_from_double(tab.dn[t]);
  for (int t = threadIdx.x; t < NG; t += blockDim.x) s_w[t] = dw_from_double(tab.w[t]);
  if (threadIdx.x == 0) {
    s_cm[0] = dw_from_double(args.c_lam);
    s_cm[1] = dw_from_double(args.c_mu);
  }
  __syncthreads();

  const int64_t warps_total = (int64_t)gridDim.x * WARPS;
  for (int64_t e = (int64_t)blockIdx.x * WARPS + warp; e < args.n_elem; e += warps_total) {
    // 1. coordinates relative to node 0; 2^k above the largest difference
    constexpr int PER = (T::NDOF + 31) / 32;
    double dif[PER];
    int emax = 0;
#pragma unroll
    for (int s = 0; s < PER; ++s) {
      const int t = lane + 32 * s;
      dif[s] = 0.0;
      if (t < T::NDOF) {
        double v, r;
        if (args.conn) {
          const int node = __ldg(args.conn + e * NN + t / 3);
          const int node0 = __ldg(args.conn + e * NN);
          v = __ldg(args.coords + 3 * (int64_t)node + (t % 3));
          r = __ldg(args.coords + 3 * (int64_t)node0 + (t % 3));
        } else {
          v = __ldg(args.xyz + e * T::NDOF + t);
          r = __ldg(args.xyz + e * T::NDOF + (t % 3));
        }
        if (!finite_bits(v)) record_error(args.status, e, AXIA_ERR_NONFINITE);
        dif[s] = v - r;
        const int be = (int)((__double_as_longlong(dif[s]) >> 52) & 0x7ff);
        emax = max(emax, be == 0x7ff ? 0 : be);
      }
    }
    emax = __reduce_max_sync(0xffffffffu, emax);
    const int k = emax == 0 ? 0 : min(max(emax - 1022, -1000), 1000);
    const double E = args.e_elem ? __ldg(args.e_elem + e) : args.e_const;
#pragma unroll
    for (int s = 0; s < PER; ++s) {
      const int t = lane + 32 * s;
      if (t < T::NDOF) Xw[t] = dw_split_scaled(dif[s], k);
    }
    __syncwarp();  // also: the previous element's c / h (J's space) are read
    // 2. J[g][q][p] = sum_a dN_a/dxi_p x_a,q (quadratic.rs:122-146 via elem.rs:175-181)
    for (int t = lane; t < NG * 9; t += 32) {
      const int g = t / 9, q = (t % 9) / 3, p = t % 3;
      const dw* dn = s_dnw + g * NN * 3;
      dw_acc s;
#pragma unroll 4
      for (int a = 0; a < NN; ++a) dw_fma(s, dn[3 * a + p], Xw[3 * a + q]);
      J[t] = dw_value(s);
    }
    __syncwarp();
    // 3. cofactor matrix b[i][j] (invert3 before the 1/det scaling, elem.rs:18-26)
    for (int t = lane; t < NG * 9; t += 32) {
      const int g = t / 9, i = (t % 9) / 3, j = t % 3;
      const dw* a = J + 9 * g;
      const int j1 = (j + 1) % 3, j2 = (j + 2) % 3, i1 = (i + 1) % 3, i2 = (i + 2) % 3;
      dw_acc s;
      dw_fma(s, a[3 * j1 + i1], a[3 * j2 + i2]);
      dw_fma(s, dw_neg(a[3 * j1 + i2]), a[3 * j2 + i1]);
      G[t] = dw_value(s);
    }
    __syncwarp();
    double vol_part = 0.0;
    for (int g = lane; g < NG; g += 32) {
      const dw* a = J + 9 * g;
      const dw* b = G + 9 * g;
      dw_acc s;
      dw_fma(s, a[0], b[0]);
      dw_fma(s, a[1], b[3]);
      dw_fma(s, a[2], b[6]);
      const dw det_s = dw_value(s);
      double det = dw_to_double(det_s);
      if (k >= -340 && k <= 340) {
        det *= pow2(3 * k);
      } else {
        const double p2k = pow2(k);
        det = det * p2k * p2k * p2k;
      }
      if (!(fabs(det) >= 1e-18)) {
        record_error(args.status, e, isfinite(det) ? AXIA_ERR_SINGULAR_JACOBIAN : AXIA_ERR_NONFINITE);
        S[g] = s_w[g];
      } else {
        if (det <= 0.0) record_error(args.status, e, AXIA_ERR_NEG_JACOBIAN);
        S[g] = dw_div(s_w[g], det_s);
      }
      vol_part += tab.w[g] * det;
    }
    if (!(__double_as_longlong(E) > 0 && __double_as_longlong(E) <= 0x7ff0000000000000ll)) {  // !(E > 0)
      if (lane == 0) record_error(args.status, e, AXIA_ERR_MATERIAL);
    }
    if (args.vol_out) {
      vol_part = warp_sum(vol_part);
      if (lane == 0) args.vol_out[e] = vol_part;
    }
    __syncwarp();  // J is read; c overwrites it
    // 4. c_a[i] = sum_p b[p][i] dN_a/dxi_p at every Gauss point
    for (int t = lane; t < NG * T::NDOF; t += 32) {
      const int g = t / T::NDOF, r = t % T::NDOF, a = r / 3, i = r % 3;
      const dw* b = G + 9 * g;
      const dw* dn = s_dnw + (g * NN + a) * 3;
      dw_acc s;
      dw_fma(s, b[i], dn[0]);
      dw_fma(s, b[3 + i], dn[1]);
      dw_fma(s, b[6 + i], dn[2]);
      C[t] = dw_value(s);
    }
    // lam and mu carry the 2^k of the scaled coordinates
    dw lam, mu;
    if (k >= -100 && k <= 100) {
      const dw Ew = dw_split_scaled(E, 0);
      lam = dw_scale(dw_mul(Ew, s_cm[0]), k);
      mu = dw_scale(dw_mul(Ew, s_cm[1]), k);
    } else {
      lam = dw_from_double(E * args.c_lam * pow2(k));
      mu = dw_from_double(E * args.c_mu * pow2(k));
    }
    __syncwarp();
    // 5. node pairs p = lane + 32 r, a <= b in row order of the upper triangle:
    // A_ab = sum_g h_a c_b^T
    double* const ke = args.ke_out + e * T::KE;
#pragma unroll 1
    for (int r = 0; r < D::NR; ++r) {
      const int p = lane + 32 * r;
      int a = 0, rem = p < T::NB ? p : 0;
      while (rem >= NN - a) {
        rem -= NN - a;
        ++a;
      }
      const int b = a + rem;
      const dw* ca = C + 3 * a;
      const dw* cb = C + 3 * b;
      dw_acc acc[9];
#pragma unroll 9
      for (int g = 0; g < NG; ++g) {
        dw hv[3], cv[3];
        const dw sg = S[g];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          hv[i] = dw_mul(sg, ca[g * T::NDOF + i]);  // h_a = (w / det) c_a
          cv[i] = cb[g * T::NDOF + i];
        }
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) dw_fma(acc[3 * i + j], hv[i], cv[j]);
      }
      if (p >= T::NB) continue;
      dw av[9];
#pragma unroll
      for (int t = 0; t < 9; ++t) av[t] = dw_value(acc[t]);
      dw_acc ts;
      dw_add(ts, av[0]);
      dw_add(ts, av[4]);
      dw_add(ts, av[8]);
      const dw tr = dw_value(ts);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          if (a == b && i > j) continue;
          dw_acc s;
          dw_fma(s, lam, av[3 * i + j]);
          dw_fma(s, mu, av[3 * j + i]);
          if (i == j) dw_fma(s, mu, tr);
          const dw v = dw_value(s);
          const int row = 3 * a + i, col = 3 * b + j;
          if (args.ke_dw) {
            dw* kw = reinterpret_cast<dw*>(ke);
            kw[row * T::NDOF + col] = v;
            kw[col * T::NDOF + row] = v;
          } else {
            const double vd = dw_to_double(v);
            ke[row * T::NDOF + col] = vd;
            ke[col * T::NDOF + row] = vd;
          }
        }
    }
  }
}
