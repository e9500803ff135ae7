// assemble.cu -- symbolic phase (node incidence, node adjacency, DOF map,
// CSR pattern of K_ff) and numeric phase (element stiffness, deterministic
// gather into K_ff with Dirichlet elimination).
//
// The reference builds K by pushing every nonzero Ke entry as a triplet in
// element order (solver/src/analysis.rs:651-668), maps the triplets to the
// independent DOFs (DofMap::reduce, solver/src/constraint.rs:138-172) and sums
// duplicates after a stable (row, col) sort (csr_from_triplets,
// solver/src/linalg.rs:10-38).  Here every row of K_ff is owned by one warp,
// which sums the contributions of the node's incident elements in ascending
// element order -- the same order the reference's stable sort keeps -- and
// writes the row once.  No atomics touch K, so the result is bitwise
// reproducible run to run.
//
// CSR pattern: all couplings of nodes that share an element (full symmetric
// storage like the reference); a block whose reference triplets are all exact
// zeros is kept as an explicit zero.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "element_dw.cuh"

// ---------------------------------------------------------------------------
// Element tables: dN/dxi at the Gauss points (hex8_shape elem.rs:158-171,
// hex20_shape quadratic.rs:36-73, hex_gauss quadratic.rs:100-120) and the
// entry/block tables of the upper triangle.
// ---------------------------------------------------------------------------
namespace {

const double kG2 = 0.5773502691896257;
const double kG3[3] = {-0.7745966692414834, 0.0, 0.7745966692414834};
const double kW3[3] = {0.5555555555555556, 0.8888888888888888, 0.5555555555555556};
const int kXi20[20][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1}, {-1, -1, 1},
                          {1, -1, 1},   {1, 1, 1},   {-1, 1, 1}, {0, -1, -1}, {1, 0, -1},
                          {0, 1, -1},   {-1, 0, -1}, {0, -1, 1}, {1, 0, 1},   {0, 1, 1},
                          {-1, 0, 1},   {-1, -1, 0}, {1, -1, 0}, {1, 1, 0},   {-1, 1, 0}};

void dshape_hex8(double xi, double eta, double zeta, double* dn) {
  for (int i = 0; i < 8; ++i) {
    double x = kXi20[i][0], e = kXi20[i][1], z = kXi20[i][2];
    dn[3 * i + 0] = 0.125 * x * (1.0 + e * eta) * (1.0 + z * zeta);
    dn[3 * i + 1] = 0.125 * e * (1.0 + x * xi) * (1.0 + z * zeta);
    dn[3 * i + 2] = 0.125 * z * (1.0 + x * xi) * (1.0 + e * eta);
  }
}

void dshape_hex20(double xi, double eta, double zeta, double* dn) {
  for (int i = 0; i < 8; ++i) {
    double x = kXi20[i][0], e = kXi20[i][1], z = kXi20[i][2];
    double a = 1.0 + x * xi, b = 1.0 + e * eta, c = 1.0 + z * zeta;
    dn[3 * i + 0] = 0.125 * x * b * c * (2.0 * x * xi + e * eta + z * zeta - 1.0);
    dn[3 * i + 1] = 0.125 * e * a * c * (x * xi + 2.0 * e * eta + z * zeta - 1.0);
    dn[3 * i + 2] = 0.125 * z * a * b * (x * xi + e * eta + 2.0 * z * zeta - 1.0);
  }
  for (int i = 8; i < 20; ++i) {
    double x = kXi20[i][0], e = kXi20[i][1], z = kXi20[i][2];
    if (x == 0) {
      dn[3 * i + 0] = 0.25 * (-2.0 * xi) * (1.0 + e * eta) * (1.0 + z * zeta);
      dn[3 * i + 1] = 0.25 * (1.0 - xi * xi) * e * (1.0 + z * zeta);
      dn[3 * i + 2] = 0.25 * (1.0 - xi * xi) * (1.0 + e * eta) * z;
    } else if (e == 0) {
      dn[3 * i + 0] = 0.25 * (1.0 - eta * eta) * x * (1.0 + z * zeta);
      dn[3 * i + 1] = 0.25 * (-2.0 * eta) * (1.0 + x * xi) * (1.0 + z * zeta);
      dn[3 * i + 2] = 0.25 * (1.0 - eta * eta) * (1.0 + x * xi) * z;
    } else {
      dn[3 * i + 0] = 0.25 * (1.0 - zeta * zeta) * x * (1.0 + e * eta);
      dn[3 * i + 1] = 0.25 * (1.0 - zeta * zeta) * (1.0 + x * xi) * e;
      dn[3 * i + 2] = 0.25 * (-2.0 * zeta) * (1.0 + x * xi) * (1.0 + e * eta);
    }
  }
}

// quadratic.rs:546-580 (tet10 in volume coordinates l1 = 1 - r - s - t, l2..l4 = r, s, t)
void dshape_tet10(double r, double s, double t, double* dn) {
  const double l1 = 1.0 - r - s - t, l2 = r, l3 = s, l4 = t;
  const double d1 = 4.0 * l1 - 1.0, d2 = 4.0 * l2 - 1.0, d3 = 4.0 * l3 - 1.0, d4 = 4.0 * l4 - 1.0;
  const double v[30] = {-d1, -d1, -d1, d2, 0.0, 0.0, 0.0, d3, 0.0, 0.0, 0.0, d4,
                        4.0 * (l1 - l2), -4.0 * l2, -4.0 * l2,
                        4.0 * l3, 4.0 * l2, 0.0,
                        -4.0 * l3, 4.0 * (l1 - l3), -4.0 * l3,
                        -4.0 * l4, -4.0 * l4, 4.0 * (l1 - l4),
                        4.0 * l4, 0.0, 4.0 * l2,
                        0.0, 4.0 * l4, 4.0 * l3};
  for (int k = 0; k < 30; ++k) dn[k] = v[k];
}

// elem.rs:221-248: linear tetrahedron, constant dN/dxi
void dshape_tet4(double* dn) {
  const double v[12] = {-1.0, -1.0, -1.0, 1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0};
  for (int k = 0; k < 12; ++k) dn[k] = v[k];
}

const double kTetA = 0.5854101966249685, kTetB = 0.1381966011250105;  // quadratic.rs:611-612

// extra.rs:64-87: linear wedge in (l1, l2) = (xi, eta), l3 = 1 - xi - eta, zeta in [-1, 1]
void dshape_wedge6(double xi, double eta, double zeta, double* dn) {
  const double l1 = xi, l2 = eta, l3 = 1.0 - xi - eta, zm = 0.5 * (1.0 - zeta), zp = 0.5 * (1.0 + zeta);
  const double v[18] = {zm, 0.0, -0.5 * l1, 0.0, zm, -0.5 * l2, -zm, -zm, -0.5 * l3,
                        zp, 0.0, 0.5 * l1,  0.0, zp, 0.5 * l2,  -zp, -zp, 0.5 * l3};
  for (int k = 0; k < 18; ++k) dn[k] = v[k];
}

// extra.rs:701-756: quadratic wedge; corner a of triangle position l_a, mid-sides
// 6..8 / 9..11 on the bottom / top edges (0-1, 1-2, 2-0), 12..14 on the vertical edges
void dshape_wedge15(double xi, double eta, double zeta, double* dn) {
  const double l[3] = {xi, eta, 1.0 - xi - eta};
  const double dl[3][2] = {{1.0, 0.0}, {0.0, 1.0}, {-1.0, -1.0}};  // d l_a / d(xi, eta)
  for (int c = 0; c < 6; ++c) {  // corners: 0.5 l (1 + s zeta)(2 l - 2 + s zeta)
    const int a = c % 3;
    const double sg = c < 3 ? -1.0 : 1.0, z = 1.0 + sg * zeta, la = l[a];
    const double dla = 0.5 * z * (4.0 * la - 2.0 + sg * zeta);
    dn[3 * c] = dla * dl[a][0];
    dn[3 * c + 1] = dla * dl[a][1];
    dn[3 * c + 2] = 0.5 * sg * la * (2.0 * la - 1.0 + 2.0 * sg * zeta);
  }
  for (int m = 0; m < 6; ++m) {  // triangle-edge mid-sides: 2 l_a l_b (1 + s zeta)
    const int a = m % 3, b = (a + 1) % 3;
    const double sg = m < 3 ? -1.0 : 1.0, z = 1.0 + sg * zeta;
    for (int p = 0; p < 2; ++p) dn[3 * (6 + m) + p] = 2.0 * z * (dl[a][p] * l[b] + l[a] * dl[b][p]);
    dn[3 * (6 + m) + 2] = 2.0 * sg * l[a] * l[b];
  }
  for (int a = 0; a < 3; ++a) {  // vertical mid-sides: l_a (1 - zeta^2)
    const double o = 1.0 - zeta * zeta;
    dn[3 * (12 + a)] = o * dl[a][0];
    dn[3 * (12 + a) + 1] = o * dl[a][1];
    dn[3 * (12 + a) + 2] = -2.0 * zeta * l[a];
  }
}

// the three triangle points of the wedge rules (extra.rs:114, 783-797)
const double kTri[3][2] = {{1.0 / 6.0, 1.0 / 6.0}, {2.0 / 3.0, 1.0 / 6.0}, {1.0 / 6.0, 2.0 / 3.0}};

}  // namespace

// dN/dxi [nn][3] at a parametric point of a C3D4 / C3D6 / C3D10 / C3D15 element
// (used by the recovery tables, which also evaluate the stress at the nodes)
void element_dshape(int nn, double r, double s, double t, double* dn) {
  if (nn == 10) dshape_tet10(r, s, t, dn);
  else if (nn == 6) dshape_wedge6(r, s, t, dn);
  else if (nn == 15) dshape_wedge15(r, s, t, dn);
  else dshape_tet4(dn);
}

namespace {

struct HostTables {
  std::vector<double> dn, w;
  std::vector<int> e0, e1, blk;
};

HostTables make_tables(int nn, int ng) {
  HostTables t;
  std::vector<double> pts;  // xi, eta, zeta, w
  if (nn == 8 && ng == 1) {
    pts = {0.0, 0.0, 0.0, 8.0};  // C3D8R: the centre, weight 8 (vol = 8 det J0, extra.rs:407)
  } else if (nn == 4) {
    pts = {0.25, 0.25, 0.25, 1.0 / 6.0};  // constant strain: one point, weight = reference volume
  } else if (nn == 10) {
    const double w = 1.0 / 24.0;  // quadratic.rs:613-614
    pts = {kTetB, kTetB, kTetB, w, kTetA, kTetB, kTetB, w, kTetB, kTetA, kTetB, w, kTetB, kTetB, kTetA, w};
  } else if (nn == 6) {  // extra.rs:114-121: triangle points x zeta = -G2, +G2, weight 1/6
    for (const auto& tp : kTri)
      for (double z : {-kG2, kG2}) pts.insert(pts.end(), {tp[0], tp[1], z, 1.0 / 6.0});
  } else if (nn == 15) {  // extra.rs:783-797: triangle points x 3-point Gauss in zeta
    for (const auto& tp : kTri)
      for (int k = 0; k < 3; ++k) pts.insert(pts.end(), {tp[0], tp[1], kG3[k], (1.0 / 6.0) * kW3[k]});
  } else if (ng == 8) {
    const double g[2] = {-kG2, kG2};
    for (double a : g)
      for (double b : g)
        for (double c : g) pts.insert(pts.end(), {a, b, c, 1.0});
  } else {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) pts.insert(pts.end(), {kG3[i], kG3[j], kG3[k], kW3[i] * kW3[j] * kW3[k]});
  }
  t.dn.resize((size_t)ng * nn * 3);
  t.w.resize(ng);
  for (int g = 0; g < ng; ++g) {
    if (nn == 8)
      dshape_hex8(pts[4 * g], pts[4 * g + 1], pts[4 * g + 2], &t.dn[(size_t)g * nn * 3]);
    else if (nn == 20)
      dshape_hex20(pts[4 * g], pts[4 * g + 1], pts[4 * g + 2], &t.dn[(size_t)g * nn * 3]);
    else
      element_dshape(nn, pts[4 * g], pts[4 * g + 1], pts[4 * g + 2], &t.dn[(size_t)g * nn * 3]);
    t.w[g] = pts[4 * g + 3];
  }
  // entries of blocks a <= b; diagonal blocks keep i <= j
  int k = 0, blk = 0;
  for (int a = 0; a < nn; ++a)
    for (int b = a; b < nn; ++b, ++blk) {
      int base = k;
      bool dg = a == b;
      t.blk.push_back(base | (dg ? 1 << 16 : 0));
      for (int i = 0; i < 3; ++i)
        for (int j = dg ? i : 0; j < 3; ++j, ++k) {
          int hi = 3 * a + i, ci = 3 * b + j;
          t.e0.push_back(hi | (ci << 8) | (i == j ? 1 << 16 : 0));
          int kT;
          if (dg) {
            kT = k;  // symmetric block
          } else {
            kT = base + 3 * j + i;
          }
          t.e1.push_back(kT | (blk << 16));
        }
    }
  return t;
}

struct DevTables {
  double* dn = nullptr;
  double* w = nullptr;
  int* e0 = nullptr;
  int* e1 = nullptr;
  int* blk = nullptr;
};

// hex8, hex20 (27 gp), hex20r (8 gp), tet4, tet10, hex8r (1 gp), wedge6,
// wedge15: one set per device, uploaded on first use under a mutex (contexts
// on different devices may be driven from different threads) and kept until
// the process exits.
constexpr int kTabDevices = 64, kTabKinds = 8;
DevTables g_tab[kTabDevices][kTabKinds];
std::mutex g_tab_mutex;

int table_index(int nn, int ng) {
  if (nn == 8 && ng == 1) return 5;
  if (nn == 4) return 3;
  if (nn == 10) return 4;
  if (nn == 6) return 6;
  if (nn == 15) return 7;
  return nn == 8 ? 0 : (ng == 27 ? 1 : 2);
}

void free_tables(DevTables& d) {
  cudaFree(d.dn);
  cudaFree(d.w);
  cudaFree(d.e0);
  cudaFree(d.e1);
  cudaFree(d.blk);
  d = DevTables{};
}

template <typename T>
cudaError_t upload(T** dst, const std::vector<T>& src) {
  cudaError_t e = cudaMalloc(dst, src.size() * sizeof(T));
  if (e == cudaSuccess) e = cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice);
  return e;
}

int ensure_tables(axia_ctx* ctx, int nn, int ng, ElemTables* out) {
  const int ti = table_index(nn, ng);
  if (ctx->device < 0 || ctx->device >= kTabDevices)
    return set_error(ctx, AXIA_ERR_INVALID_ARG, "device index out of range for the element tables");
  std::lock_guard<std::mutex> lock(g_tab_mutex);
  DevTables& d = g_tab[ctx->device][ti];
  if (!d.blk) {  // blk is uploaded last: set only when the whole set is on the device
    const HostTables h = make_tables(nn, ng);
    DevTables t;
    cudaError_t e = upload(&t.dn, h.dn);
    if (e == cudaSuccess) e = upload(&t.w, h.w);
    if (e == cudaSuccess) e = upload(&t.e0, h.e0);
    if (e == cudaSuccess) e = upload(&t.e1, h.e1);
    if (e == cudaSuccess) e = upload(&t.blk, h.blk);
    if (e != cudaSuccess) {
      free_tables(t);
      return set_error(ctx, AXIA_ERR_CUDA, std::string("element table upload: ") + cudaGetErrorString(e));
    }
    d = t;
  }
  out->dn = d.dn;
  out->w = d.w;
  out->e0 = d.e0;
  out->e1 = d.e1;
  out->blk = d.blk;
  return AXIA_OK;
}

// DW: the double-word Gauss loop (element_dw.cuh) instead of the FP64 one
template <int NN, int NG, int WARPS, bool DW = false>
int launch_element_ke(axia_ctx* ctx, const ElemArgs& args) {
  ElemTables tab;
  AXIA_TRY(ensure_tables(ctx, NN, NG, &tab));
  size_t smem;
  void (*kern)(ElemArgs, ElemTables);
  if constexpr (DW && NN == 20) {
    smem = element_dw_pair_smem_bytes<NN, NG>(WARPS);
    kern = element_ke_dw_pair_kernel<NN, NG, WARPS>;
  } else if constexpr (DW) {
    smem = element_dw_smem_bytes<NN, NG>(WARPS);
    kern = element_ke_dw_kernel<NN, NG, WARPS>;
  } else {
    smem = element_smem_bytes<NN, NG>(WARPS);
    kern = element_ke_kernel<NN, NG, WARPS>;
  }
  AXIA_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  AXIA_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, WARPS * 32, smem));
  if (per_sm < 1) return set_error(ctx, AXIA_ERR_CUDA, "element kernel does not fit on an SM");
  int64_t need = (args.n_elem + WARPS - 1) / WARPS;
  int64_t grid = std::min<int64_t>(need, (int64_t)per_sm * ctx->sm_count);
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, WARPS * 32, smem, ctx->stream>>>(args, tab);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  return AXIA_OK;
}

}  // namespace

// dN/dxi and weights of the Gauss points of (nn, ng) in device memory
int element_tables_for(axia_ctx* ctx, int nn, int ng, const double** dn, const double** w) {
  ElemTables t;
  AXIA_TRY(ensure_tables(ctx, nn, ng, &t));
  *dn = t.dn;
  *w = t.w;
  return AXIA_OK;
}

// Runs the element kernel for nn / reduced on args (device pointers).
int run_hex8r_hourglass(axia_ctx* ctx, const ElemArgs& args);
int run_hex8i_condense(axia_ctx* ctx, const ElemArgs& args, const double* dn_tab);

// true when run_element_ke runs a double-word kernel for this kind: C3D8
// (element_ke_dw_kernel), C3D20 and C3D20R (element_ke_dw_pair_kernel).
bool element_uses_dw(const axia_ctx* ctx, int nn, int reduced) {
  return !ctx->element_fp64 && ((nn == 8 && reduced == 0) || nn == 20);
}

// nn = 8: reduced 1 = C3D8R (centre point + hourglass), 2 = C3D8I (incompatible modes)
int run_element_ke(axia_ctx* ctx, int nn, int reduced, const ElemArgs& args) {
  if (args.n_elem == 0) return AXIA_OK;
  if (nn == 8 && reduced == 1) {
    AXIA_TRY((launch_element_ke<8, 1, 8>(ctx, args)));
    return run_hex8r_hourglass(ctx, args);
  }
  if (nn == 8 && reduced == 2) {
    AXIA_TRY((launch_element_ke<8, 8, 8>(ctx, args)));
    ElemTables tab;
    AXIA_TRY(ensure_tables(ctx, 8, 8, &tab));
    return run_hex8i_condense(ctx, args, tab.dn);
  }
  const bool dw = element_uses_dw(ctx, nn, reduced);
  if (nn == 8) return dw ? launch_element_ke<8, 8, 8, true>(ctx, args) : launch_element_ke<8, 8, 8>(ctx, args);
  if (nn == 20 && !reduced)
    return dw ? launch_element_ke<20, 27, 14, true>(ctx, args) : launch_element_ke<20, 27, 4>(ctx, args);
  if (nn == 20 && reduced)
    return dw ? launch_element_ke<20, 8, 8, true>(ctx, args) : launch_element_ke<20, 8, 4>(ctx, args);
  if (nn == 4) return launch_element_ke<4, 1, 8>(ctx, args);
  if (nn == 10) return launch_element_ke<10, 4, 8>(ctx, args);
  if (nn == 6) return launch_element_ke<6, 6, 8>(ctx, args);
  if (nn == 15) return launch_element_ke<15, 9, 4>(ctx, args);
  return set_error(ctx, AXIA_ERR_INVALID_ARG, "nn must be 4, 6, 8, 10, 15 or 20");
}

// ---------------------------------------------------------------------------
// Symbolic kernels
// ---------------------------------------------------------------------------
__global__ void k_count_incidence(int64_t n_items, int nn, const int32_t* conn, int64_t n_nodes,
                                  int64_t* cnt, DevStatus* st) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n_items;
       t += (int64_t)gridDim.x * blockDim.x) {
    int node = conn[t];
    if (node < 0 || node >= n_nodes) {
      record_error(st, t / nn, AXIA_ERR_INVALID_ARG);
      continue;
    }
    atomicAdd((unsigned long long*)&cnt[node], 1ull);
  }
}

__global__ void k_fill_incidence(int64_t n_items, int nn, const int32_t* conn, const int64_t* ptr,
                                 int32_t* fill, int32_t* ne) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n_items;
       t += (int64_t)gridDim.x * blockDim.x) {
    int node = conn[t];
    int pos = atomicAdd(&fill[node], 1);
    int64_t e = t / nn;
    int la = (int)(t % nn);
    ne[ptr[node] + pos] = (int32_t)(e * 32 + la);
  }
}

// insertion sort of every node's incidence list: ascending element, then local index
__global__ void k_sort_incidence(int64_t n_nodes, const int64_t* ptr, int32_t* ne) {
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < n_nodes;
       a += (int64_t)gridDim.x * blockDim.x) {
    int64_t b = ptr[a], e = ptr[a + 1];
    for (int64_t i = b + 1; i < e; ++i) {
      int32_t v = ne[i];
      int64_t j = i - 1;
      while (j >= b && ne[j] > v) {
        ne[j + 1] = ne[j];
        --j;
      }
      ne[j + 1] = v;
    }
  }
}

// Adjacency of node a: sorted unique nodes of its incident elements.
// mode 0 counts (cnt[a]), mode 1 writes adj[ptr[a] ...].  One warp per node;
// candidates staged in shared memory (cap per warp = cap).
// Sorted distinct neighbours of one node from its m <= 32 K candidates, in
// registers: element i = 32 k + lane of a bitonic network over 32 K slots
// (padding INT_MAX), partners within a lane swapped in registers, across
// lanes exchanged by shuffles.  mode 0 returns the count, mode 1 also writes
// the list (ascending) to out.
template <int K>
__device__ __forceinline__ int warp_sorted_unique(int m, int nn, const int32_t* conn, const int32_t* ne_b0, int lane,
                                                  int mode, int32_t* out) {
  int v[K];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const int t = 32 * k + lane;
    v[k] = t < m ? conn[(int64_t)(ne_b0[t / nn] >> 5) * nn + (t % nn)] : INT_MAX;
  }
#pragma unroll
  for (int size = 2; size <= 32 * K; size <<= 1) {
#pragma unroll
    for (int j = size >> 1; j > 0; j >>= 1) {
      if (j >= 32) {
        const int J = j >> 5;
#pragma unroll
        for (int k = 0; k < K; ++k) {
          if (k & J) continue;
          const bool asc = ((32 * k + lane) & size) == 0;
          const int lo = min(v[k], v[k | J]), hi = max(v[k], v[k | J]);
          v[k] = asc ? lo : hi;
          v[k | J] = asc ? hi : lo;
        }
      } else {
#pragma unroll
        for (int k = 0; k < K; ++k) {
          const int o = __shfl_xor_sync(0xffffffffu, v[k], j);
          const bool asc = ((32 * k + lane) & size) == 0;
          const bool lower = (lane & j) == 0;
          v[k] = (lower == asc) ? min(v[k], o) : max(v[k], o);
        }
      }
    }
  }
  int count = 0;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    int prev = __shfl_up_sync(0xffffffffu, v[k], 1);
    const int last_prev = k > 0 ? __shfl_sync(0xffffffffu, v[k > 0 ? k - 1 : 0], 31) : INT_MIN;
    if (lane == 0) prev = last_prev;
    const bool f = v[k] != INT_MAX && v[k] != prev;
    const unsigned bal = __ballot_sync(0xffffffffu, f);
    if (mode == 1 && f) out[count + __popc(bal & ((1u << lane) - 1u))] = v[k];
    count += __popc(bal);
  }
  return count;
}

__global__ void k_adjacency(int64_t n_nodes, int nn, const int32_t* conn, const int64_t* ne_ptr,
                            const int32_t* ne, int cap, int mode, int64_t* cnt, const int64_t* adj_ptr,
                            int32_t* adj, DevStatus* st) {
  extern __shared__ int32_t s_cand[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  int32_t* cand = s_cand + (size_t)warp * 2 * cap;
  int32_t* first = cand + cap;
  for (int64_t a = (int64_t)blockIdx.x * wpb + warp; a < n_nodes; a += (int64_t)gridDim.x * wpb) {
    int64_t b0 = ne_ptr[a], b1 = ne_ptr[a + 1];
    int m = (int)(b1 - b0) * nn;
    if (m > cap) {
      if (lane == 0) record_error(st, a, AXIA_ERR_TOO_LARGE);
      continue;
    }
    if (m <= 256) {  // register sort (warp-uniform branch: m is the node's)
      int32_t* out = mode == 1 ? adj + adj_ptr[a] : nullptr;
      int c;
      if (m <= 64)
        c = warp_sorted_unique<2>(m, nn, conn, ne + b0, lane, mode, out);
      else if (m <= 128)
        c = warp_sorted_unique<4>(m, nn, conn, ne + b0, lane, mode, out);
      else
        c = warp_sorted_unique<8>(m, nn, conn, ne + b0, lane, mode, out);
      if (mode == 0 && lane == 0) cnt[a] = c;
      continue;
    }
    for (int t = lane; t < m; t += 32) {
      int32_t code = ne[b0 + t / nn];
      cand[t] = conn[(int64_t)(code >> 5) * nn + (t % nn)];
    }
    __syncwarp();
    for (int i = lane; i < m; i += 32) {
      int v = cand[i], f = 1;
      for (int j = 0; j < i; ++j)
        if (cand[j] == v) {
          f = 0;
          break;
        }
      first[i] = f;
    }
    __syncwarp();
    int my_count = 0;
    for (int i = lane; i < m; i += 32) {
      if (!first[i]) continue;
      ++my_count;
      if (mode == 1) {
        int v = cand[i], pos = 0;
        for (int j = 0; j < m; ++j) pos += (first[j] && cand[j] < v) ? 1 : 0;
        adj[adj_ptr[a] + pos] = v;
      }
    }
    my_count = warp_sum(my_count);
    if (mode == 0 && lane == 0) cnt[a] = my_count;
    __syncwarp();
  }
}

// free[d] = !prescribed[d] && node attached (analysis.rs:2283-2330 pins isolated nodes)
__global__ void k_free_flags(int64_t ndof, const uint8_t* presc, const int64_t* inc_cnt, int64_t* flag) {
  for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < ndof;
       d += (int64_t)gridDim.x * blockDim.x)
    flag[d] = (!presc[d] && inc_cnt[d / 3] > 0) ? 1 : 0;
}

__global__ void k_ind_of(int64_t ndof, const int64_t* flag, const int64_t* scan, int32_t* ind_of) {
  for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < ndof;
       d += (int64_t)gridDim.x * blockDim.x)
    ind_of[d] = flag[d] ? (int32_t)scan[d] : -1;
}

// per node: free-column offset of every adjacency block and the row length
__global__ void k_row_layout(int64_t n_nodes, const int64_t* adj_ptr, const int32_t* adj,
                             const int32_t* ind_of, int32_t* adj_off, int32_t* rowlen) {
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < n_nodes;
       a += (int64_t)gridDim.x * blockDim.x) {
    int run = 0;
    for (int64_t s = adj_ptr[a]; s < adj_ptr[a + 1]; ++s) {
      int b = adj[s];
      adj_off[s] = run;
      run += (ind_of[3 * (int64_t)b] >= 0) + (ind_of[3 * (int64_t)b + 1] >= 0) + (ind_of[3 * (int64_t)b + 2] >= 0);
    }
    rowlen[a] = run;
  }
}

__global__ void k_row_counts(int64_t ndof, const int32_t* ind_of, const int32_t* rowlen, int64_t* cnt) {
  for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < ndof;
       d += (int64_t)gridDim.x * blockDim.x) {
    int r = ind_of[d];
    if (r >= 0) cnt[r] = rowlen[d / 3];
  }
}

__global__ void k_to_i32(int64_t n, const int64_t* in, int32_t* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (int32_t)in[i];
}

// first free index of node b (free DOFs of a node are consecutive)
__device__ __forceinline__ int first_free(const int32_t* ind_of, int b) {
  int c = ind_of[3 * b];
  if (c < 0) c = ind_of[3 * b + 1];
  if (c < 0) c = ind_of[3 * b + 2];
  return c;
}

// column indices of every free row, warp per node
// padded block-row lengths: each row rounded up to a multiple of 4 blocks
__global__ void k_quad_counts(int64_t n_nodes, const int64_t* adj_ptr, int64_t* qcnt) {
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a <= n_nodes; a += (int64_t)gridDim.x * blockDim.x)
    qcnt[a] = a < n_nodes ? ((adj_ptr[a + 1] - adj_ptr[a] + 3) & ~(int64_t)3) : 0;
}

// padded block columns: the row's adjacency, then the row's own node as filler
__global__ void k_quad_fill(int64_t n_nodes, const int64_t* adj_ptr, const int32_t* adj, const int64_t* qptr,
                            int32_t* qadj) {
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < n_nodes; a += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s0 = adj_ptr[a], len = adj_ptr[a + 1] - s0, q0 = qptr[a], qlen = qptr[a + 1] - q0;
    for (int64_t s = 0; s < qlen; ++s) qadj[q0 + s] = s < len ? adj[s0 + s] : (int32_t)a;
  }
}

__global__ void k_fill_columns(int64_t n_nodes, const int64_t* adj_ptr, const int32_t* adj,
                               const int32_t* adj_off, const int32_t* ind_of, const int32_t* rowptr,
                               int32_t* col) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  for (int64_t a = (int64_t)blockIdx.x * wpb + warp; a < n_nodes; a += (int64_t)gridDim.x * wpb) {
    int64_t s0 = adj_ptr[a];
    int nadj = (int)(adj_ptr[a + 1] - s0);
    for (int i = 0; i < 3; ++i) {
      int r = ind_of[3 * a + i];
      if (r < 0) continue;
      int64_t rs = rowptr[r];
      for (int t = lane; t < 3 * nadj; t += 32) {
        int s = t / 3, j = t % 3;
        int b = adj[s0 + s];
        int c = ind_of[3 * (int64_t)b + j];
        if (c >= 0) col[rs + adj_off[s0 + s] + (c - first_free(ind_of, b))] = c;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Symmetric node-block form (AXIA_ASM_SYM32): structure from the sorted node
// adjacency.  Row a keeps its blocks b >= a (the adjacency's tail, starting at
// the diagonal) as upper blocks, padded to an even count, and lists its
// neighbours b < a with the position of K_ba among row b's upper blocks.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int lower_bound_i32(const int32_t* v, int n, int key) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (v[mid] < key) lo = mid + 1; else hi = mid;
  }
  return lo;
}

__global__ void k_sym_counts(int64_t n_nodes, const int64_t* adj_ptr, const int32_t* adj, int64_t* ucnt,
                             int64_t* lcnt) {
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a <= n_nodes; a += (int64_t)gridDim.x * blockDim.x) {
    if (a == n_nodes) {
      ucnt[a] = lcnt[a] = 0;
      continue;
    }
    const int64_t s0 = adj_ptr[a];
    const int len = (int)(adj_ptr[a + 1] - s0);
    const int first = lower_bound_i32(adj + s0, len, (int)a);
    ucnt[a] = (len - first + 1) & ~1;
    lcnt[a] = first;
  }
}

__global__ void k_sym_lower(int64_t n_nodes, const int64_t* adj_ptr, const int32_t* adj, const int64_t* uptr,
                            const int64_t* lptr, int2* low) {
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < n_nodes; a += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s0 = adj_ptr[a], l0 = lptr[a];
    const int nl = (int)(lptr[a + 1] - l0);
    for (int k = 0; k < nl; ++k) {
      const int b = adj[s0 + k];  // b < a: the sorted adjacency's head
      const int64_t t0 = adj_ptr[b];
      const int blen = (int)(adj_ptr[b + 1] - t0);
      const int first_b = lower_bound_i32(adj + t0, blen, b);
      const int at = lower_bound_i32(adj + t0, blen, (int)a);
      low[l0 + k] = make_int2(b, (int)(uptr[b] + (at - first_b)));
    }
  }
}

// pad blocks of the upper rows: zero values, the row's own node as column
__global__ void k_sym_pad(int64_t n_nodes, const int64_t* adj_ptr, const int32_t* adj, const int64_t* uptr,
                          float* uval) {
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < n_nodes; a += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s0 = adj_ptr[a];
    const int len = (int)(adj_ptr[a + 1] - s0);
    const int nu = len - lower_bound_i32(adj + s0, len, (int)a);
    for (int64_t k = uptr[a] + nu; k < uptr[a + 1]; ++k) {
      for (int c = 0; c < 9; ++c) uval[10 * k + c] = 0.f;
      uval[10 * k + 9] = __int_as_float((int)a);
    }
  }
}

// ---------------------------------------------------------------------------
// Numeric gather: warp per node, contributions of incident elements summed in
// ascending element order into a shared-memory block row, then written as up
// to three CSR rows of K_ff (free columns) and K_fp u0 (prescribed columns).
// ---------------------------------------------------------------------------
struct GatherArgs {
  int64_t n_nodes;
  int nn;
  const int32_t* conn;
  const int64_t* ne_ptr;
  const int32_t* ne;
  const int64_t* adj_ptr;
  const int32_t* adj;
  const int32_t* adj_off;
  const int32_t* ind_of;
  const int32_t* rowptr;
  const double* ke;
  const double* u0;
  int any_u0;
  int max_adj;
  int warp_stride;   // bytes of shared memory per warp
  double* val;        // CSR FP64 values (null: not assembled)
  float* val32;       // CSR FP32 values (null: not assembled)
  double* diag;
  double* dinv;
  float* dinv32;
  double* kfu0;
  double* bval64;     // node-block values [9][nb] (null: not assembled)
  float* bval32;
  float* bval32lo;    // fl32(K64 - K32) [9][nb] (null: not assembled)
  double* bdinv64;    // full-DOF 1/diag, 1 on prescribed DOFs
  float* bdinv32;
  const int32_t* qptr;  // padded node-block row starts
  int64_t nb;           // padded block count (plane stride)
  float* uval;          // symmetric FP32 form [nbu][10] (null: not assembled)
  const int32_t* uptr;  // its upper-block row starts
  int ke_dw;            // ke holds double words (element_ke_dw_kernel): sums in double words
};

// incident elements whose column slots are looked up at once (x nodes per
// element <= GATHER_SLOTS), and the Ke values per lane of one element's row block
constexpr int GATHER_SLOTS = 64;
constexpr int GATHER_VPL = 6;  // ceil(3 * 60 / 32): C3D20

// DWK: the Ke scratch holds double words; each K entry is then summed in a
// compensated double-word accumulator (dword.cuh) on the FP32 pipe and
// rounded once to FP64 (and to FP32 for the FP32 forms), instead of one FP64
// add per element contribution.
// NNT: nodes per element when fixed at compile time (8, 20), 0 for g.nn.
template <bool DWK, int NNT>
__global__ void k_gather(GatherArgs g) {
  extern __shared__ __align__(16) unsigned char s_gather[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  const int nn = NNT ? NNT : g.nn, ndof_e = 3 * nn, ke_size = ndof_e * ndof_e;
  const int per = 3 * ndof_e, nv = (per + 31) / 32;
  const int batch = max(1, GATHER_SLOTS / nn);
  // the lane's values of an element's row block: element node c / 3 and the
  // entry i * 3 + c % 3 of the 3 x 3 block they add to (fixed per lane)
  int v_node[GATHER_VPL], v_ent[GATHER_VPL];
#pragma unroll
  for (int m = 0; m < GATHER_VPL; ++m) {
    const int t = lane + 32 * m;
    const int i = t / ndof_e, c = t - i * ndof_e;
    v_node[m] = c / 3;
    v_ent[m] = i * 3 + c % 3;
  }
  unsigned char* base = s_gather + (size_t)warp * g.warp_stride;
  double* acc = (double*)base;                                   // [max_adj][9]
  dw_acc* acw = (dw_acc*)base;                                   // the same, DWK
  int32_t* s_adj = (int32_t*)(base + (size_t)g.max_adj * 72);    // [max_adj]
  int32_t* s_slot = s_adj + g.max_adj;                           // [GATHER_SLOTS]
  int32_t* s_code = s_slot + GATHER_SLOTS;                       // [GATHER_SLOTS]
  for (int64_t a = (int64_t)blockIdx.x * wpb + warp; a < g.n_nodes; a += (int64_t)gridDim.x * wpb) {
    const int64_t s0 = g.adj_ptr[a];
    const int nadj = (int)(g.adj_ptr[a + 1] - s0);
    for (int t = lane; t < nadj; t += 32) s_adj[t] = g.adj[s0 + t];
    for (int t = lane; t < nadj * 9; t += 32) acc[t] = 0.0;
    __syncwarp();
    const int64_t kend = g.ne_ptr[a + 1];
    for (int64_t k0 = g.ne_ptr[a]; k0 < kend; k0 += batch) {
      const int nbat = kend - k0 < batch ? (int)(kend - k0) : batch;
      // element codes and the column slots of their nodes, all at once
      for (int t = lane; t < nbat; t += 32) s_code[t] = g.ne[k0 + t];
      __syncwarp();
      for (int t = lane; t < nbat * nn; t += 32) {
        const int b = g.conn[(int64_t)(s_code[t / nn] >> 5) * nn + t % nn];
        int lo = 0, hi = nadj - 1;
        while (lo < hi) {
          int mid = (lo + hi) >> 1;
          if (s_adj[mid] < b) lo = mid + 1; else hi = mid;
        }
        s_slot[t] = lo;
      }
      __syncwarp();
      // element by element in ascending element order, the next element's
      // row block loaded while the current one is summed
      double cur[GATHER_VPL], nxt[GATHER_VPL];
      auto load = [&](int j, double* v) {
        const int32_t code = s_code[j];
        const double* rowblk = g.ke + (int64_t)(code >> 5) * ke_size + (int64_t)(3 * (code & 31)) * ndof_e;
#pragma unroll
        for (int m = 0; m < GATHER_VPL; ++m) {
          const int t = lane + 32 * m;
          v[m] = (m < nv && t < per) ? __ldcs(rowblk + t) : 0.0;
        }
      };
      load(0, cur);
      for (int j = 0; j < nbat; ++j) {
        if (j + 1 < nbat) load(j + 1, nxt);
#pragma unroll
        for (int m = 0; m < GATHER_VPL; ++m) {
          const int t = lane + 32 * m;
          if (m < nv && t < per) {
            const int idx = s_slot[j * nn + v_node[m]] * 9 + v_ent[m];
            if constexpr (DWK) {
              const long long bits = __double_as_longlong(cur[m]);
              dw_acc q = acw[idx];
              dw_add(q, dw{__int_as_float((int)bits), __int_as_float((int)(bits >> 32))});
              acw[idx] = q;
            } else {
              acc[idx] += cur[m];
            }
          }
        }
        __syncwarp();
#pragma unroll
        for (int m = 0; m < GATHER_VPL; ++m) cur[m] = nxt[m];
      }
    }
    // the summed entry idx in FP64, in FP32 and the FP32 low part fl32(v64 - v32)
    auto kval3 = [&](int idx, double& v64, float& v32, float& lo) {
      if constexpr (DWK) {
        const dw v = dw_value(acw[idx]);
        v64 = dw_to_double(v);
        v32 = v.h;
        lo = v.l;
      } else {
        v64 = acc[idx];
        v32 = (float)v64;
        lo = g.bval32lo ? (float)(v64 - f32_to_f64_exact(v32)) : 0.f;
      }
    };
    auto kval = [&](int idx, double& v64, float& v32) {
      float lo;
      kval3(idx, v64, v32, lo);
    };
    // K_ff in CSR, and K_fp u0 -- skipped for a node-block-only assembly
    // without prescribed values (the diagonal is then written below)
    const bool csr_pass = g.val || g.val32 || g.any_u0;
    for (int i = 0; csr_pass && i < 3; ++i) {
      const int r = g.ind_of[3 * a + i];
      if (r < 0) continue;
      const int64_t rs = g.rowptr[r];
      double kf = 0.0;
      for (int t = lane; t < 3 * nadj; t += 32) {
        const int s = t / 3, j = t % 3;
        const int b = s_adj[s];
        double v;
        float v32;
        kval(s * 9 + i * 3 + j, v, v32);
        const int c = g.ind_of[3 * (int64_t)b + j];
        if (c >= 0) {
          const int64_t pos = rs + g.adj_off[s0 + s] + (c - first_free(g.ind_of, b));
          if (g.val) g.val[pos] = v;
          if (g.val32) g.val32[pos] = v32;
          if (c == r) {
            g.diag[r] = v;
            const double di = fabs(v) > 1e-30 ? 1.0 / v : 1.0;  // linalg.rs:218-219 guard
            g.dinv[r] = di;
            if (g.dinv32) g.dinv32[r] = (float)di;
          }
        } else if (g.any_u0) {
          const double u0 = g.u0[3 * (int64_t)b + j];
          if (u0 != 0.0) kf = fma(v, u0, kf);
        }
      }
      if (g.any_u0) {
        kf = warp_sum(kf);
        if (lane == 0) g.kfu0[r] = kf;
      }
    }
    if (g.uval) {
      // symmetric form: the blocks b >= a of the row (sorted adjacency tail), 9 values + column
      const int first_up = lower_bound_i32(s_adj, nadj, (int)a);
      const int nu = nadj - first_up;
      const int64_t u0 = g.uptr[a];
      for (int t = lane; t < 10 * nu; t += 32) {
        const int k = t / 10, c = t - 10 * k, s = first_up + k;
        const int b = s_adj[s];
        float v;
        if (c < 9) {
          const int i = c / 3, j = c % 3;
          const bool fi = g.ind_of[3 * a + i] >= 0, fj = g.ind_of[3 * (int64_t)b + j] >= 0;
          double v64;
          float v32;
          kval(s * 9 + c, v64, v32);
          v = (fi && fj) ? v32 : ((b == a && i == j) ? 1.f : 0.f);
        } else {
          v = __int_as_float(b);
        }
        g.uval[10 * (u0 + k) + c] = v;
      }
    }
    if (g.bval64 || g.bval32 || g.uval) {
      // node-block form: free-free entries of K, a unit diagonal on prescribed
      // DOFs; lanes take the row's blocks s, each all 9 entries (for every
      // entry the lanes write consecutive blocks of one value plane)
      bool fi[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) fi[i] = g.ind_of[3 * a + i] >= 0;
      const int64_t q0 = g.qptr[a];
      for (int s = lane; s < nadj; s += 32) {
        const int b = s_adj[s];
        bool fj[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) fj[j] = g.ind_of[3 * (int64_t)b + j] >= 0;
#pragma unroll
        for (int ij = 0; ij < 9; ++ij) {
          const int i = ij / 3, j = ij % 3;
          double v;
          float v32, lo;
          kval3(s * 9 + ij, v, v32, lo);
          if (!(fi[i] && fj[j])) {
            const bool dg = (b == a) && (i == j);
            v = dg ? 1.0 : 0.0;
            v32 = dg ? 1.f : 0.f;
            lo = 0.f;
          }
          const int64_t pos = (int64_t)ij * g.nb + q0 + s;
          if (g.bval64) g.bval64[pos] = v;
          if (g.bval32) g.bval32[pos] = v32;
          if (g.bval32lo) g.bval32lo[pos] = lo;
        }
      }
      // 1 / diagonal, one division per lane on lanes 0..2 (linalg.rs:218-219 guard)
      if (lane < 3) {
        const int i = lane;
        const int self = lower_bound_i32(s_adj, nadj, (int)a);
        double v;
        float v32;
        kval(self * 9 + 4 * i, v, v32);
        const bool f = g.ind_of[3 * a + i] >= 0;
        double di;
        float di32;
        if constexpr (DWK) {  // 1 / d in double words (48 bits) on the FP32 pipe
          const dw d = dw_value(acw[self * 9 + 4 * i]);
          const dw q = f && fabsf(d.h) > 1e-30f ? dw_div(dw{1.f, 0.f}, d) : dw{1.f, 0.f};
          di = dw_to_double(q);
          di32 = q.h;
        } else {
          di = f ? (fabs(v) > 1e-30 ? 1.0 / v : 1.0) : 1.0;
          di32 = (float)di;
        }
        if (g.bdinv64) g.bdinv64[3 * a + i] = di;
        if (g.bdinv32) g.bdinv32[3 * a + i] = di32;
        if (!csr_pass && f) {  // the K_ff diagonal the CSR pass would have written
          const int r = g.ind_of[3 * a + i];
          g.diag[r] = v;
          g.dinv[r] = di;
          if (g.dinv32) g.dinv32[r] = di32;
        }
      }
    }
    __syncwarp();
  }
}

int run_gather(axia_ctx* ctx, GatherArgs args) {
  size_t per_warp = (size_t)args.max_adj * 9 * sizeof(double) + (size_t)(args.max_adj + 2 * GATHER_SLOTS) * 4;
  per_warp = (per_warp + 15) & ~(size_t)15;
  if (per_warp > 200 * 1024) return set_error(ctx, AXIA_ERR_TOO_LARGE, "node adjacency too large for the gather");
  int warps = 8;
  while (warps > 1 && per_warp * warps > 200 * 1024) warps /= 2;
  args.warp_stride = (int)per_warp;
  size_t stride = per_warp;
  size_t smem = stride * warps;
  void (*kern)(GatherArgs);
  if (args.nn == 8)
    kern = args.ke_dw ? k_gather<true, 8> : k_gather<false, 8>;
  else if (args.nn == 20)
    kern = args.ke_dw ? k_gather<true, 20> : k_gather<false, 20>;
  else
    kern = args.ke_dw ? k_gather<true, 0> : k_gather<false, 0>;
  AXIA_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  AXIA_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, warps * 32, smem));
  if (per_sm < 1) per_sm = 1;
  int64_t need = (args.n_nodes + warps - 1) / warps;
  int64_t grid = std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)per_sm * ctx->sm_count));
  kern<<<(unsigned)grid, warps * 32, smem, ctx->stream>>>(args);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  return AXIA_OK;
}

// ---------------------------------------------------------------------------
// Host drivers
// ---------------------------------------------------------------------------
static unsigned grid_for(int64_t n, int threads, int sm_count) {
  int64_t g = (n + threads - 1) / threads;
  g = std::min<int64_t>(g, (int64_t)sm_count * 32);
  return (unsigned)std::max<int64_t>(g, 1);
}

// prescribed DOFs from the BC list, last BC wins (analysis.rs:556-565): the
// largest BC index per DOF, then its value
__global__ void k_bc_winner(int64_t n_bc, const int64_t* bc_dof, int* win) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_bc; k += (int64_t)gridDim.x * blockDim.x)
    atomicMax(win + bc_dof[k], (int)k);
}
__global__ void k_bc_apply(int64_t ndof, const int* win, const double* bc_val, uint8_t* presc, double* u0,
                           int* any_u0) {
  for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < ndof; d += (int64_t)gridDim.x * blockDim.x) {
    const int k = win[d];
    const double v = k >= 0 ? bc_val[k] : 0.0;
    presc[d] = k >= 0;
    u0[d] = v;
    if (v != 0.0) *any_u0 = 1;
  }
}

// largest ptr[a + 1] - ptr[a] over a < n
__global__ void k_max_len(int64_t n, const int64_t* ptr, int* out) {
  int m = 0;
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < n; a += (int64_t)gridDim.x * blockDim.x)
    m = max(m, (int)(ptr[a + 1] - ptr[a]));
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

static int device_max_len(axia_ctx* ctx, int64_t n, const int64_t* d_ptr, int* result) {
  int* d_m = nullptr;
  AXIA_TRY(dev_alloc(ctx, &d_m, 1));
  AXIA_CUDA(ctx, cudaMemsetAsync(d_m, 0, sizeof(int), ctx->stream));
  k_max_len<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, ctx->sm_count * 8)), 256, 0,
              ctx->stream>>>(n, d_ptr, d_m);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaMemcpyAsync(result, d_m, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  dev_release(ctx, d_m);
  return AXIA_OK;
}

int symbolic_setup(axia_ctx* ctx, int64_t n_bc, const int64_t* d_bc_dof, const double* d_bc_val) {
  const int64_t n_nodes = ctx->n_nodes, n_elem = ctx->n_elem, nn = ctx->nn, ndof = ctx->ndof;
  const int64_t n_items = n_elem * nn;
  cudaStream_t s = ctx->stream;
  int64_t *d_cnt = nullptr, *d_ne_ptr = nullptr;
  int32_t* d_fill = nullptr;
  AXIA_TRY(dev_alloc(ctx, &d_cnt, n_nodes + 1));
  AXIA_TRY(dev_alloc(ctx, &d_ne_ptr, n_nodes + 1));
  AXIA_TRY(dev_alloc(ctx, &d_fill, n_nodes));
  AXIA_CUDA(ctx, cudaMemsetAsync(d_cnt, 0, (n_nodes + 1) * sizeof(int64_t), s));
  AXIA_CUDA(ctx, cudaMemsetAsync(d_fill, 0, n_nodes * sizeof(int32_t), s));
  k_count_incidence<<<grid_for(n_items, 256, ctx->sm_count), 256, 0, s>>>(n_items, (int)nn, ctx->d_conn,
                                                                           n_nodes, d_cnt, ctx->d_status);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  DevStatus hs;
  AXIA_TRY(read_dev_status(ctx, &hs));
  if (hs.first_error != ~0ull)
    return set_error(ctx, AXIA_ERR_INVALID_ARG,
                     "element " + std::to_string(hs.first_error >> 8) + " names a node outside 0..n_nodes-1");
  int64_t total = 0;
  AXIA_TRY(device_exclusive_scan(ctx, d_cnt, d_ne_ptr, n_nodes + 1, &total));
  // per-node incidence maximum (for the adjacency candidate cap)
  int max_inc = 0;
  AXIA_TRY(device_max_len(ctx, n_nodes, d_ne_ptr, &max_inc));
  ctx->max_inc = max_inc;
  AXIA_TRY(dev_alloc(ctx, &ctx->d_ne, n_items));
  k_fill_incidence<<<grid_for(n_items, 256, ctx->sm_count), 256, 0, s>>>(n_items, (int)nn, ctx->d_conn, d_ne_ptr,
                                                                          d_fill, ctx->d_ne);
  ctx->launches++;
  k_sort_incidence<<<grid_for(n_nodes, 128, ctx->sm_count), 128, 0, s>>>(n_nodes, d_ne_ptr, ctx->d_ne);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  // adjacency
  const int cap = std::max<int>(32, max_inc * (int)nn);
  if (cap > 4096) return set_error(ctx, AXIA_ERR_TOO_LARGE, "a node touches too many elements");
  int64_t *d_adj_cnt = nullptr, *d_adj_ptr = nullptr;
  AXIA_TRY(dev_alloc(ctx, &d_adj_cnt, n_nodes + 1));
  AXIA_TRY(dev_alloc(ctx, &d_adj_ptr, n_nodes + 1));
  AXIA_CUDA(ctx, cudaMemsetAsync(d_adj_cnt, 0, (n_nodes + 1) * sizeof(int64_t), s));
  int wpb = 4;
  size_t smem_adj = (size_t)wpb * 2 * cap * sizeof(int32_t);
  AXIA_CUDA(ctx, cudaFuncSetAttribute(k_adjacency, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_adj));
  unsigned g_adj = grid_for(n_nodes, wpb, ctx->sm_count);
  k_adjacency<<<g_adj, wpb * 32, smem_adj, s>>>(n_nodes, (int)nn, ctx->d_conn, d_ne_ptr, ctx->d_ne, cap, 0, d_adj_cnt,
                                                nullptr, nullptr, ctx->d_status);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  int64_t n_adj = 0;
  AXIA_TRY(device_exclusive_scan(ctx, d_adj_cnt, d_adj_ptr, n_nodes + 1, &n_adj));
  ctx->n_adj = n_adj;
  AXIA_TRY(dev_alloc(ctx, &ctx->d_adj, n_adj));
  AXIA_TRY(dev_alloc(ctx, &ctx->d_adj_off, n_adj));
  k_adjacency<<<g_adj, wpb * 32, smem_adj, s>>>(n_nodes, (int)nn, ctx->d_conn, d_ne_ptr, ctx->d_ne, cap, 1, nullptr,
                                                d_adj_ptr, ctx->d_adj, ctx->d_status);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  AXIA_TRY(device_max_len(ctx, n_nodes, d_adj_ptr, &ctx->max_adj));
  // DOF map
  uint8_t* d_presc = nullptr;
  int64_t *d_flag = nullptr, *d_scan = nullptr;
  AXIA_TRY(dev_alloc(ctx, &d_presc, ndof));
  AXIA_TRY(dev_alloc(ctx, &d_flag, ndof + 1));
  AXIA_TRY(dev_alloc(ctx, &d_scan, ndof + 1));
  AXIA_TRY(dev_alloc(ctx, &ctx->d_u0, ndof));
  AXIA_TRY(dev_alloc(ctx, &ctx->d_ind_of, ndof));
  {
    int *d_win = nullptr, *d_any = nullptr;
    AXIA_TRY(dev_alloc(ctx, &d_win, ndof));
    AXIA_TRY(dev_alloc(ctx, &d_any, 1));
    AXIA_CUDA(ctx, cudaMemsetAsync(d_win, 0xff, ndof * sizeof(int), s));  // -1: no BC
    AXIA_CUDA(ctx, cudaMemsetAsync(d_any, 0, sizeof(int), s));
    if (n_bc > 0)
      k_bc_winner<<<grid_for(n_bc, 256, ctx->sm_count), 256, 0, s>>>(n_bc, d_bc_dof, d_win);
    k_bc_apply<<<grid_for(ndof, 256, ctx->sm_count), 256, 0, s>>>(ndof, d_win, d_bc_val, d_presc, ctx->d_u0, d_any);
    ctx->launches += 2;
    int any = 0;
    AXIA_CUDA(ctx, cudaMemcpyAsync(&any, d_any, sizeof(int), cudaMemcpyDeviceToHost, s));
    AXIA_CUDA(ctx, cudaStreamSynchronize(s));
    ctx->any_u0 = any != 0;
    dev_release(ctx, d_win);
    dev_release(ctx, d_any);
  }
  AXIA_CUDA(ctx, cudaMemsetAsync(d_flag + ndof, 0, sizeof(int64_t), s));
  k_free_flags<<<grid_for(ndof, 256, ctx->sm_count), 256, 0, s>>>(ndof, d_presc, d_cnt, d_flag);
  ctx->launches++;
  int64_t n_free = 0;
  AXIA_TRY(device_exclusive_scan(ctx, d_flag, d_scan, ndof + 1, &n_free));
  k_ind_of<<<grid_for(ndof, 256, ctx->sm_count), 256, 0, s>>>(ndof, d_flag, d_scan, ctx->d_ind_of);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  ctx->n_free = n_free;
  // row layout
  AXIA_TRY(dev_alloc(ctx, &ctx->d_node_rowlen, n_nodes));
  k_row_layout<<<grid_for(n_nodes, 128, ctx->sm_count), 128, 0, s>>>(n_nodes, d_adj_ptr, ctx->d_adj, ctx->d_ind_of,
                                                                     ctx->d_adj_off, ctx->d_node_rowlen);
  ctx->launches++;
  int64_t *d_rcnt = nullptr, *d_rptr = nullptr;
  AXIA_TRY(dev_alloc(ctx, &d_rcnt, n_free + 1));
  AXIA_TRY(dev_alloc(ctx, &d_rptr, n_free + 1));
  AXIA_CUDA(ctx, cudaMemsetAsync(d_rcnt, 0, (n_free + 1) * sizeof(int64_t), s));
  k_row_counts<<<grid_for(ndof, 256, ctx->sm_count), 256, 0, s>>>(ndof, ctx->d_ind_of, ctx->d_node_rowlen, d_rcnt);
  ctx->launches++;
  int64_t nnz = 0;
  AXIA_TRY(device_exclusive_scan(ctx, d_rcnt, d_rptr, n_free + 1, &nnz));
  if (nnz >= (int64_t)INT32_MAX)
    return set_error(ctx, AXIA_ERR_TOO_LARGE, "nnz(K_ff) = " + std::to_string(nnz) + " exceeds 2^31-1");
  ctx->nnz = nnz;
  AXIA_TRY(dev_alloc(ctx, &ctx->d_rowptr, n_free + 1));
  k_to_i32<<<grid_for(n_free + 1, 256, ctx->sm_count), 256, 0, s>>>(n_free + 1, d_rptr, ctx->d_rowptr);
  ctx->launches++;
  // the column indices of K_ff (nnz int32) are filled on first use by a CSR
  // assembly or export (ensure_csr_columns): the node-block solves never read them
  AXIA_CUDA(ctx, cudaGetLastError());
  AXIA_CUDA(ctx, cudaStreamSynchronize(s));
  AXIA_TRY(read_dev_status(ctx, &hs));
  if (hs.first_error != ~0ull)
    return set_error(ctx, AXIA_ERR_TOO_LARGE, "node " + std::to_string(hs.first_error >> 8) +
                                                  ": adjacency candidate list above the cap");
  // int32 copy of the block-row pointers for the node-block kernels
  AXIA_TRY(dev_alloc(ctx, &ctx->d_adj_ptr32, n_nodes + 1));
  k_to_i32<<<grid_for(n_nodes + 1, 256, ctx->sm_count), 256, 0, s>>>(n_nodes + 1, d_adj_ptr, ctx->d_adj_ptr32);
  ctx->launches++;
  // padded block rows of the node-block form
  {
    int64_t *d_qcnt = nullptr, *d_qptr64 = nullptr;
    AXIA_TRY(dev_alloc(ctx, &d_qcnt, n_nodes + 1));
    AXIA_TRY(dev_alloc(ctx, &d_qptr64, n_nodes + 1));
    k_quad_counts<<<grid_for(n_nodes + 1, 256, ctx->sm_count), 256, 0, s>>>(n_nodes, d_adj_ptr, d_qcnt);
    ctx->launches++;
    int64_t nbq = 0;
    AXIA_TRY(device_exclusive_scan(ctx, d_qcnt, d_qptr64, n_nodes + 1, &nbq));
    if (nbq >= (int64_t)INT32_MAX) return set_error(ctx, AXIA_ERR_TOO_LARGE, "node blocks exceed 2^31-1");
    ctx->nbq = nbq;
    AXIA_TRY(dev_alloc(ctx, &ctx->d_qptr, n_nodes + 1));
    AXIA_TRY(dev_alloc(ctx, &ctx->d_qadj, (size_t)std::max<int64_t>(nbq, 4)));
    k_to_i32<<<grid_for(n_nodes + 1, 256, ctx->sm_count), 256, 0, s>>>(n_nodes + 1, d_qptr64, ctx->d_qptr);
    k_quad_fill<<<grid_for(n_nodes, 256, ctx->sm_count), 256, 0, s>>>(n_nodes, d_adj_ptr, ctx->d_adj, d_qptr64,
                                                                       ctx->d_qadj);
    ctx->launches += 2;
    AXIA_CUDA(ctx, cudaGetLastError());
    AXIA_CUDA(ctx, cudaStreamSynchronize(s));
    dev_release(ctx, d_qcnt);
    dev_release(ctx, d_qptr64);
  }
  // keep the 64-bit pointers for the gather
  dev_release(ctx, ctx->d_ne_ptr);
  dev_release(ctx, ctx->d_adj_ptr);
  ctx->d_ne_ptr = d_ne_ptr;
  ctx->d_adj_ptr = d_adj_ptr;
  dev_release(ctx, d_cnt);
  dev_release(ctx, d_fill);
  dev_release(ctx, d_adj_cnt);
  dev_release(ctx, d_presc);
  dev_release(ctx, d_flag);
  dev_release(ctx, d_scan);
  dev_release(ctx, d_rcnt);
  dev_release(ctx, d_rptr);
  return AXIA_OK;
}

// Structure of the symmetric FP32 node-block form, built on first use per mesh:
// upper-block row starts (even counts), pad blocks, lower lists.
static int ensure_sym_structure(axia_ctx* ctx) {
  if (ctx->d_uval) return AXIA_OK;
  cudaStream_t s = ctx->stream;
  const int64_t n_nodes = ctx->n_nodes;
  int64_t *d_ucnt = nullptr, *d_lcnt = nullptr, *d_uptr64 = nullptr, *d_lptr64 = nullptr;
  AXIA_TRY(dev_alloc(ctx, &d_ucnt, n_nodes + 1));
  AXIA_TRY(dev_alloc(ctx, &d_lcnt, n_nodes + 1));
  AXIA_TRY(dev_alloc(ctx, &d_uptr64, n_nodes + 1));
  AXIA_TRY(dev_alloc(ctx, &d_lptr64, n_nodes + 1));
  k_sym_counts<<<grid_for(n_nodes + 1, 256, ctx->sm_count), 256, 0, s>>>(n_nodes, ctx->d_adj_ptr, ctx->d_adj, d_ucnt,
                                                                        d_lcnt);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  int64_t nbu = 0, nbl = 0;
  AXIA_TRY(device_exclusive_scan(ctx, d_ucnt, d_uptr64, n_nodes + 1, &nbu));
  AXIA_TRY(device_exclusive_scan(ctx, d_lcnt, d_lptr64, n_nodes + 1, &nbl));
  if (nbu >= (int64_t)INT32_MAX / 10 || nbl >= (int64_t)INT32_MAX)
    return set_error(ctx, AXIA_ERR_TOO_LARGE, "symmetric node-block form exceeds 32-bit positions");
  AXIA_TRY(dev_alloc(ctx, &ctx->d_uptr, n_nodes + 1));
  AXIA_TRY(dev_alloc(ctx, &ctx->d_lptr, n_nodes + 1));
  AXIA_TRY(dev_alloc(ctx, &ctx->d_uval, (size_t)std::max<int64_t>(10 * nbu, 20)));
  AXIA_TRY(dev_alloc(ctx, &ctx->d_low, (size_t)std::max<int64_t>(nbl, 1)));
  k_to_i32<<<grid_for(n_nodes + 1, 256, ctx->sm_count), 256, 0, s>>>(n_nodes + 1, d_uptr64, ctx->d_uptr);
  k_to_i32<<<grid_for(n_nodes + 1, 256, ctx->sm_count), 256, 0, s>>>(n_nodes + 1, d_lptr64, ctx->d_lptr);
  k_sym_lower<<<grid_for(n_nodes, 128, ctx->sm_count), 128, 0, s>>>(n_nodes, ctx->d_adj_ptr, ctx->d_adj, d_uptr64,
                                                                    d_lptr64, ctx->d_low);
  k_sym_pad<<<grid_for(n_nodes, 256, ctx->sm_count), 256, 0, s>>>(n_nodes, ctx->d_adj_ptr, ctx->d_adj, d_uptr64,
                                                                  ctx->d_uval);
  ctx->launches += 4;
  AXIA_CUDA(ctx, cudaGetLastError());
  AXIA_CUDA(ctx, cudaStreamSynchronize(s));
  dev_release(ctx, d_ucnt);
  dev_release(ctx, d_lcnt);
  dev_release(ctx, d_uptr64);
  dev_release(ctx, d_lptr64);
  ctx->nbu = nbu;
  ctx->nbl = nbl;
  return AXIA_OK;
}

// Column indices of K_ff in CSR, built once per mesh when a CSR form is first
// assembled or exported (warp per node from the node adjacency and the DOF map).
int ensure_csr_columns(axia_ctx* ctx) {
  if (ctx->d_col || ctx->nnz == 0) return AXIA_OK;
  AXIA_TRY(dev_alloc(ctx, &ctx->d_col, (size_t)ctx->nnz));
  k_fill_columns<<<grid_for(ctx->n_nodes, 8, ctx->sm_count), 256, 0, ctx->stream>>>(
      ctx->n_nodes, ctx->d_adj_ptr, ctx->d_adj, ctx->d_adj_off, ctx->d_ind_of, ctx->d_rowptr, ctx->d_col);
  ctx->launches++;
  AXIA_CUDA(ctx, cudaGetLastError());
  return AXIA_OK;
}

int numeric_assemble(axia_ctx* ctx, int flags) {
  cudaStream_t s = ctx->stream;
  const bool csr64 = flags & AXIA_ASM_CSR64, csr32 = flags & AXIA_ASM_CSR32;
  const bool bsr64 = flags & AXIA_ASM_BSR64, bsr32 = flags & AXIA_ASM_BSR32;
  const bool sym32 = flags & AXIA_ASM_SYM32;
  const bool bsr32lo = bsr32 && (flags & AXIA_ASM_BSR32LO);
  if (sym32) AXIA_TRY(ensure_sym_structure(ctx));
  if (csr64 || csr32) AXIA_TRY(ensure_csr_columns(ctx));
  const int64_t kesz = (int64_t)9 * ctx->nn * ctx->nn;
  if (ctx->ke_elems < (size_t)(ctx->n_elem * kesz)) {
    AXIA_TRY(dev_alloc(ctx, &ctx->d_ke, (size_t)(ctx->n_elem * kesz)));
    ctx->ke_elems = (size_t)(ctx->n_elem * kesz);
  }
  AXIA_TRY(reset_dev_status(ctx));
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  for (auto& e : ev) AXIA_CUDA(ctx, cudaEventCreate(&e));
  struct EvGuard {
    cudaEvent_t* e;
    ~EvGuard() {
      for (int k = 0; k < 3; ++k)
        if (e[k]) cudaEventDestroy(e[k]);
    }
  } ev_guard{ev};
  cudaEventRecord(ev[0], s);
  ElemArgs ea{};
  ea.n_elem = ctx->n_elem;
  ea.conn = ctx->d_conn;
  ea.coords = ctx->d_coords;
  ea.xyz = nullptr;
  ea.e_elem = ctx->d_e;
  ea.e_const = 0.0;
  ea.c_lam = ctx->nu / ((1.0 + ctx->nu) * (1.0 - 2.0 * ctx->nu));
  ea.c_mu = 1.0 / (2.0 * (1.0 + ctx->nu));
  ea.ke_out = ctx->d_ke;
  ea.vol_out = nullptr;
  ea.status = ctx->d_status;
  ea.ke_dw = element_uses_dw(ctx, ctx->nn, ctx->reduced) ? 1 : 0;
  ctx->ke_dw = ea.ke_dw != 0;
  AXIA_TRY(run_element_ke(ctx, ctx->nn, ctx->reduced, ea));
  cudaEventRecord(ev[1], s);
  if (csr64 && !ctx->d_val) AXIA_TRY(dev_alloc(ctx, &ctx->d_val, ctx->nnz));
  if (csr32 && !ctx->d_val32) AXIA_TRY(dev_alloc(ctx, &ctx->d_val32, ctx->nnz));
  if (!ctx->d_diag) AXIA_TRY(dev_alloc(ctx, &ctx->d_diag, ctx->n_free));
  if (!ctx->d_dinv) AXIA_TRY(dev_alloc(ctx, &ctx->d_dinv, ctx->n_free));
  if (csr32 && !ctx->d_dinv32) AXIA_TRY(dev_alloc(ctx, &ctx->d_dinv32, ctx->n_free));
  if (!ctx->d_kfu0) AXIA_TRY(dev_alloc(ctx, &ctx->d_kfu0, ctx->n_free));
  // padding blocks stay zero: they are cleared once here and never written
  if (bsr64 && !ctx->d_bval64) {
    AXIA_TRY(dev_alloc(ctx, &ctx->d_bval64, (size_t)(9 * ctx->nbq)));
    AXIA_CUDA(ctx, cudaMemsetAsync(ctx->d_bval64, 0, (size_t)(9 * ctx->nbq) * sizeof(double), s));
  }
  if (bsr32 && !ctx->d_bval32) {
    AXIA_TRY(dev_alloc(ctx, &ctx->d_bval32, (size_t)(9 * ctx->nbq)));
    AXIA_CUDA(ctx, cudaMemsetAsync(ctx->d_bval32, 0, (size_t)(9 * ctx->nbq) * sizeof(float), s));
  }
  if (bsr32lo && !ctx->d_bval32lo) {
    AXIA_TRY(dev_alloc(ctx, &ctx->d_bval32lo, (size_t)(9 * ctx->nbq)));
    AXIA_CUDA(ctx, cudaMemsetAsync(ctx->d_bval32lo, 0, (size_t)(9 * ctx->nbq) * sizeof(float), s));
  }
  if ((bsr64 || bsr32 || sym32) && !ctx->d_bdinv64) AXIA_TRY(dev_alloc(ctx, &ctx->d_bdinv64, (size_t)ctx->ndof));
  if ((bsr32 || sym32) && !ctx->d_bdinv32) AXIA_TRY(dev_alloc(ctx, &ctx->d_bdinv32, (size_t)ctx->ndof));
  AXIA_CUDA(ctx, cudaMemsetAsync(ctx->d_kfu0, 0, ctx->n_free * sizeof(double), s));
  GatherArgs g{};
  g.n_nodes = ctx->n_nodes;
  g.nn = ctx->nn;
  g.conn = ctx->d_conn;
  g.ne_ptr = ctx->d_ne_ptr;
  g.ne = ctx->d_ne;
  g.adj_ptr = ctx->d_adj_ptr;
  g.adj = ctx->d_adj;
  g.adj_off = ctx->d_adj_off;
  g.ind_of = ctx->d_ind_of;
  g.rowptr = ctx->d_rowptr;
  g.ke = ctx->d_ke;
  g.u0 = ctx->d_u0;
  g.any_u0 = ctx->any_u0 ? 1 : 0;
  g.max_adj = std::max(ctx->max_adj, 1);
  g.val = csr64 ? ctx->d_val : nullptr;
  g.val32 = csr32 ? ctx->d_val32 : nullptr;
  g.diag = ctx->d_diag;
  g.dinv = ctx->d_dinv;
  g.dinv32 = csr32 ? ctx->d_dinv32 : nullptr;
  g.kfu0 = ctx->d_kfu0;
  g.bval64 = bsr64 ? ctx->d_bval64 : nullptr;
  g.bval32 = bsr32 ? ctx->d_bval32 : nullptr;
  g.bval32lo = bsr32lo ? ctx->d_bval32lo : nullptr;
  g.bdinv64 = (bsr64 || bsr32 || sym32) ? ctx->d_bdinv64 : nullptr;
  g.bdinv32 = (bsr32 || sym32) ? ctx->d_bdinv32 : nullptr;
  g.qptr = ctx->d_qptr;
  g.nb = ctx->nbq;
  g.uval = sym32 ? ctx->d_uval : nullptr;
  g.uptr = ctx->d_uptr;
  g.ke_dw = ctx->ke_dw ? 1 : 0;
  // the gather's interval also holds the first-use allocations and clears above
  // (none after the first assembly of a mesh)
  AXIA_TRY(run_gather(ctx, g));
  cudaEventRecord(ev[2], s);
  AXIA_CUDA(ctx, cudaStreamSynchronize(s));
  {
    float m1 = 0.f, m2 = 0.f;
    cudaEventElapsedTime(&m1, ev[0], ev[1]);
    cudaEventElapsedTime(&m2, ev[1], ev[2]);
    ctx->ms_element = m1;
    ctx->ms_gather = m2;
  }
  DevStatus hs;
  AXIA_TRY(read_dev_status(ctx, &hs));
  ctx->have_csr64 = ctx->have32 = ctx->have_bsr64 = ctx->have_bsr32 = ctx->have_sym32 = ctx->have_bsr32lo = false;
  ctx->assembled = false;
  if (hs.first_error != ~0ull) {
    int code = (int)(hs.first_error & 0xff);
    long long idx = (long long)(hs.first_error >> 8);
    static const char* names[] = {"", "invalid argument", "singular Jacobian (degenerate element)",
                                  "negative Jacobian determinant", "invalid material (E <= 0)"};
    std::string what = code < 5 ? names[code] : (code == AXIA_ERR_NONFINITE ? "non-finite value" : "error");
    ctx->last_bad = idx;
    return set_error(ctx, code, "element " + std::to_string(idx) + ": " + what);
  }
  ctx->have_csr64 = csr64;
  ctx->have32 = csr32;
  ctx->have_bsr64 = bsr64;
  ctx->have_bsr32 = bsr32;
  ctx->have_bsr32lo = bsr32lo;
  ctx->have_sym32 = sym32;
  ctx->assembled = true;
  ctx->assemble_gen++;
  return AXIA_OK;
}
