// noalloc.cu -- batched element stiffness without any device allocation.
//
// axia_gpu_element_ke_noalloc is axia_gpu_element_ke for callers that must
// not allocate GPU memory: hosts whose device memory belongs to another
// allocator (a caching allocator or a fixed budget they may not exceed), and
// latency-critical loops where cudaMalloc / cudaFree, which can synchronize
// the device, are not acceptable.  It needs no context either.
//
// Its device memory is one file-scope __device__ array (kScratchBytes, held by
// every GPU that loads the library until the process exits): the element
// tables, the status word and the staging of coordinates, moduli, Ke and
// volumes.  The element kernels are the ones the context path runs by default
// (double words for C3D8, the FP64 loop for C3D20 / C3D20R).  Host code only ever passes the array's device address, which the
// first call on each device looks up with cudaGetSymbolAddress (with that
// device current) and caches; that first call should come before any stream
// capture.  Every call reuses the array: the status word is cleared at the
// start of each call, and calls that overlap on the GPU would race (calls in
// one process are serialized by a host mutex).  The cached address and tables
// belong to the CUDA context that was current at the first call: calls after
// cudaDeviceReset (or any teardown of the primary context) are not supported.
#include <mutex>

#include "element_dw.cuh"

namespace {

constexpr int64_t kMaxElemHex8 = 2048;   // C3D8 elements per call
constexpr int64_t kMaxElemHex20 = 512;   // C3D20 / C3D20R elements per call
constexpr size_t kScratchBytes = 16u << 20;
constexpr size_t kTableBase = 4096;       // element tables: 3 kinds x 64 KiB
constexpr size_t kTableStride = 64u << 10;
constexpr size_t kDataBase = kTableBase + 3 * kTableStride;

__device__ __align__(256) unsigned char g_scratch[kScratchBytes];

struct DeviceState {
  unsigned char* base = nullptr;  // device address of g_scratch on this device
  bool ready = false;
};
DeviceState g_state[64];
std::mutex g_mutex;

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// dN/dxi of the 8 / 20 node hexahedron (hex8_shape elem.rs:158-171,
// hex20_shape quadratic.rs:36-73) at (xi, eta, zeta) into dn[3*NN]
void hex_dshape(int nn, double xi, double eta, double zeta, double* dn) {
  static const int P[20][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1}, {-1, -1, 1},
                               {1, -1, 1},   {1, 1, 1},   {-1, 1, 1}, {0, -1, -1}, {1, 0, -1},
                               {0, 1, -1},   {-1, 0, -1}, {0, -1, 1}, {1, 0, 1},   {0, 1, 1},
                               {-1, 0, 1},   {-1, -1, 0}, {1, -1, 0}, {1, 1, 0},   {-1, 1, 0}};
  for (int i = 0; i < nn; ++i) {
    const double x = P[i][0], e = P[i][1], z = P[i][2];
    const double a = 1.0 + x * xi, b = 1.0 + e * eta, c = 1.0 + z * zeta;
    if (nn == 8) {
      dn[3 * i] = 0.125 * x * b * c;
      dn[3 * i + 1] = 0.125 * e * a * c;
      dn[3 * i + 2] = 0.125 * z * a * b;
    } else if (i < 8) {
      dn[3 * i] = 0.125 * x * b * c * (2.0 * x * xi + e * eta + z * zeta - 1.0);
      dn[3 * i + 1] = 0.125 * e * a * c * (x * xi + 2.0 * e * eta + z * zeta - 1.0);
      dn[3 * i + 2] = 0.125 * z * a * b * (x * xi + e * eta + 2.0 * z * zeta - 1.0);
    } else if (x == 0) {
      dn[3 * i] = -0.5 * xi * b * c;
      dn[3 * i + 1] = 0.25 * (1.0 - xi * xi) * e * c;
      dn[3 * i + 2] = 0.25 * (1.0 - xi * xi) * b * z;
    } else if (e == 0) {
      dn[3 * i] = 0.25 * (1.0 - eta * eta) * x * c;
      dn[3 * i + 1] = -0.5 * eta * a * c;
      dn[3 * i + 2] = 0.25 * (1.0 - eta * eta) * a * z;
    } else {
      dn[3 * i] = 0.25 * (1.0 - zeta * zeta) * x * b;
      dn[3 * i + 1] = 0.25 * (1.0 - zeta * zeta) * a * e;
      dn[3 * i + 2] = -0.5 * zeta * a * b;
    }
  }
}

// Element tables of one kind written into host staging arrays, laid out as
// dn | w | e0 | e1 | blk (the ElemTables the kernel reads), then copied into
// the scratch at kTableBase + kind * kTableStride.
struct TableView {
  size_t off_dn, off_w, off_e0, off_e1, off_blk, bytes;
};

TableView table_layout(int nn, int ng) {
  const int ne = 9 * nn * (nn - 1) / 2 + 6 * nn, nb = nn * (nn + 1) / 2;
  TableView v;
  v.off_dn = 0;
  v.off_w = align256(v.off_dn + sizeof(double) * ng * nn * 3);
  v.off_e0 = align256(v.off_w + sizeof(double) * ng);
  v.off_e1 = align256(v.off_e0 + sizeof(int) * ne);
  v.off_blk = align256(v.off_e1 + sizeof(int) * ne);
  v.bytes = v.off_blk + sizeof(int) * nb;
  return v;
}

int upload_tables(unsigned char* dev_base, int kind, int nn, int ng) {
  alignas(256) static unsigned char host[kTableStride];
  const TableView v = table_layout(nn, ng);
  double* dn = reinterpret_cast<double*>(host + v.off_dn);
  double* w = reinterpret_cast<double*>(host + v.off_w);
  int* e0 = reinterpret_cast<int*>(host + v.off_e0);
  int* e1 = reinterpret_cast<int*>(host + v.off_e1);
  int* blk = reinterpret_cast<int*>(host + v.off_blk);
  const double g2 = 0.5773502691896257;
  const double g3[3] = {-0.7745966692414834, 0.0, 0.7745966692414834};
  const double w3[3] = {0.5555555555555556, 0.8888888888888888, 0.5555555555555556};
  int g = 0;
  if (ng == 8) {
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j)
        for (int k = 0; k < 2; ++k, ++g) {
          hex_dshape(nn, i ? g2 : -g2, j ? g2 : -g2, k ? g2 : -g2, dn + 3 * nn * g);
          w[g] = 1.0;
        }
  } else {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k, ++g) {
          hex_dshape(nn, g3[i], g3[j], g3[k], dn + 3 * nn * g);
          w[g] = w3[i] * w3[j] * w3[k];
        }
  }
  int ent = 0, b = 0;
  for (int a = 0; a < nn; ++a)
    for (int c = a; c < nn; ++c, ++b) {
      const int base = ent;
      const bool dg = a == c;
      blk[b] = base | (dg ? 1 << 16 : 0);
      for (int i = 0; i < 3; ++i)
        for (int j = dg ? i : 0; j < 3; ++j, ++ent) {
          e0[ent] = (3 * a + i) | ((3 * c + j) << 8) | (i == j ? 1 << 16 : 0);
          e1[ent] = (dg ? ent : base + 3 * j + i) | (b << 16);
        }
    }
  if (cudaMemcpy(dev_base + kTableBase + kind * kTableStride, host, v.bytes, cudaMemcpyHostToDevice) != cudaSuccess)
    return AXIA_ERR_CUDA;
  return AXIA_OK;
}

int ensure_device(int device, unsigned char** base) {
  if (device < 0 || device >= 64) return AXIA_ERR_INVALID_ARG;
  DeviceState& s = g_state[device];
  if (!s.ready) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return AXIA_ERR_CUDA;
    s.base = static_cast<unsigned char*>(p);
    if (upload_tables(s.base, 0, 8, 8) != AXIA_OK) return AXIA_ERR_CUDA;
    if (upload_tables(s.base, 1, 20, 27) != AXIA_OK) return AXIA_ERR_CUDA;
    if (upload_tables(s.base, 2, 20, 8) != AXIA_OK) return AXIA_ERR_CUDA;
    s.ready = true;
  }
  *base = s.base;
  return AXIA_OK;
}

template <int NN, int NG, int WARPS>
int launch(unsigned char* base, int kind, const ElemArgs& args) {
  const TableView v = table_layout(NN, NG);
  unsigned char* t = base + kTableBase + kind * kTableStride;
  ElemTables tab;
  tab.dn = reinterpret_cast<const double*>(t + v.off_dn);
  tab.w = reinterpret_cast<const double*>(t + v.off_w);
  tab.e0 = reinterpret_cast<const int*>(t + v.off_e0);
  tab.e1 = reinterpret_cast<const int*>(t + v.off_e1);
  tab.blk = reinterpret_cast<const int*>(t + v.off_blk);
  // the context path's default kernels: double words for C3D8 (per-entry
  // lanes) and for C3D20(R) (node-pair lanes)
  size_t smem;
  void (*kern)(ElemArgs, ElemTables);
  if constexpr (NN == 8) {
    smem = element_dw_smem_bytes<NN, NG>(WARPS);
    kern = element_ke_dw_kernel<NN, NG, WARPS>;
  } else {
    smem = element_dw_pair_smem_bytes<NN, NG>(WARPS);
    kern = element_ke_dw_pair_kernel<NN, NG, WARPS>;
  }
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return AXIA_ERR_CUDA;
  int device = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&device) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, WARPS * 32, smem) != cudaSuccess || per_sm < 1)
    return AXIA_ERR_CUDA;
  const int64_t need = (args.n_elem + WARPS - 1) / WARPS;
  const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)per_sm * sms));
  kern<<<(unsigned)grid, WARPS * 32, smem, 0>>>(args, tab);
  return cudaGetLastError() == cudaSuccess ? AXIA_OK : AXIA_ERR_CUDA;
}

}  // namespace

extern "C" AXIA_API int32_t axia_gpu_element_ke_noalloc(int32_t nn, int32_t reduced, int64_t n_elem,
                                                        const double* xyz, const double* e, double nu, double* ke,
                                                        double* vol, int64_t* bad_elem) {
  if (bad_elem) *bad_elem = -1;
  // C3D8, C3D20 and C3D20R only: the C3D8R / C3D8I arms (reduced = 1 / 2 with
  // nn = 8) need the hourglass and condensation kernels of the context path,
  // and any other `reduced` would silently pick a different element.
  if (nn != 8 && nn != 20) return AXIA_ERR_INVALID_ARG;
  if ((nn == 8 && reduced != 0) || (nn == 20 && reduced != 0 && reduced != 1)) return AXIA_ERR_INVALID_ARG;
  const int64_t max_elem = nn == 8 ? kMaxElemHex8 : kMaxElemHex20;
  if (n_elem < 0) return AXIA_ERR_INVALID_ARG;
  if (n_elem > max_elem) return AXIA_ERR_TOO_LARGE;
  if (n_elem > 0 && (!xyz || !e || !ke)) return AXIA_ERR_INVALID_ARG;
  if (nu >= 0.5 || nu <= -1.0 || !(nu == nu)) return AXIA_ERR_MATERIAL;  // d_iso_3d, elem.rs:42-44
  if (n_elem == 0) return AXIA_OK;
  std::lock_guard<std::mutex> lock(g_mutex);
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) return AXIA_ERR_CUDA;
  unsigned char* base = nullptr;
  int st = ensure_device(device, &base);
  if (st != AXIA_OK) return st;
  const int64_t nd = 3 * (int64_t)nn, kesz = nd * nd;
  // data region: status | xyz | e | ke | vol
  size_t off = kDataBase;
  DevStatus* d_status = reinterpret_cast<DevStatus*>(base + off);
  off = align256(off + sizeof(DevStatus));
  double* d_xyz = reinterpret_cast<double*>(base + off);
  off = align256(off + sizeof(double) * n_elem * nd);
  double* d_e = reinterpret_cast<double*>(base + off);
  off = align256(off + sizeof(double) * n_elem);
  double* d_ke = reinterpret_cast<double*>(base + off);
  off = align256(off + sizeof(double) * n_elem * kesz);
  double* d_vol = reinterpret_cast<double*>(base + off);
  off = align256(off + sizeof(double) * n_elem);
  if (off > kScratchBytes) return AXIA_ERR_TOO_LARGE;
  DevStatus clean;
  clean.first_error = ~0ull;
  clean.timeout = 0;
  clean.pad = 0;
  if (cudaMemcpy(d_status, &clean, sizeof(clean), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(d_xyz, xyz, sizeof(double) * n_elem * nd, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(d_e, e, sizeof(double) * n_elem, cudaMemcpyHostToDevice) != cudaSuccess)
    return AXIA_ERR_CUDA;
  ElemArgs a{};
  a.n_elem = n_elem;
  a.conn = nullptr;
  a.coords = nullptr;
  a.xyz = d_xyz;
  a.e_elem = d_e;
  a.c_lam = nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
  a.c_mu = 1.0 / (2.0 * (1.0 + nu));
  a.ke_out = d_ke;
  a.vol_out = d_vol;
  a.status = d_status;
  if (nn == 8)
    st = launch<8, 8, 8>(base, 0, a);
  else if (!reduced)
    st = launch<20, 27, 14>(base, 1, a);
  else
    st = launch<20, 8, 8>(base, 2, a);
  if (st != AXIA_OK) return st;
  DevStatus hs;
  if (cudaMemcpy(ke, d_ke, sizeof(double) * n_elem * kesz, cudaMemcpyDeviceToHost) != cudaSuccess ||
      (vol && cudaMemcpy(vol, d_vol, sizeof(double) * n_elem, cudaMemcpyDeviceToHost) != cudaSuccess) ||
      cudaMemcpy(&hs, d_status, sizeof(hs), cudaMemcpyDeviceToHost) != cudaSuccess)
    return AXIA_ERR_CUDA;
  if (hs.first_error != ~0ull) {
    if (bad_elem) *bad_elem = (int64_t)(hs.first_error >> 8);
    return (int32_t)(hs.first_error & 0xff);
  }
  return AXIA_OK;
}
