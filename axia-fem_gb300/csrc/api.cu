// api.cu -- the extern "C" entry points declared in include/axia_gpu.h.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

#include "element.cuh"
#include "solver.cuh"

int symbolic_setup(axia_ctx* ctx, int64_t n_bc, const int64_t* d_bc_dof, const double* d_bc_val);
int numeric_assemble(axia_ctx* ctx, int flags);
int ensure_csr_columns(axia_ctx* ctx);
int bsr_solve(axia_ctx* ctx, const double* d_f, double* d_u, const axia_solve_opts* opts, axia_solve_info* info);
int bsr_spmv_device(axia_ctx* ctx, bool fp32, const void* x, void* y, int lanes_req, int vec_req);
int sym_spmv_device(axia_ctx* ctx, const float* x, float* y, int lanes_req);
int element_energy(axia_ctx* ctx, const double* d_u, const double* d_v, double* d_s);
int simp_modulus(axia_ctx* ctx, const double* d_rho, double pexp, double e0);
int simp_gradient(axia_ctx* ctx, const double* d_rho, const double* d_s, double pexp, double e0, double* d_g);
int device_dot(axia_ctx* ctx, const double* a, const double* b, int64_t n, double* out);
void multimesh_release(axia_ctx* ctx);
int batch_block_solve(axia_ctx* ctx, int nrhs, const double* d_F, double* d_U, const axia_solve_opts* opts,
                      axia_solve_info* info, double* rel_res);
int batch_solve(axia_ctx* ctx, int nrhs, const double* d_F, double* d_U, const axia_solve_opts* opts,
                axia_solve_info* info, double* rel_res);
int run_element_ke(axia_ctx* ctx, int nn, int reduced, const ElemArgs& args);
struct PcgOut;
int pcg_solve(axia_ctx* ctx, const axia_solve_opts* opts, axia_solve_info* info);
int ensure_pcg_state(axia_ctx* ctx);
int build_rhs(axia_ctx* ctx, const double* d_f);
int reconstruct(axia_ctx* ctx, double* d_u);
int true_residual(axia_ctx* ctx, double* out);
int prepare_solve(axia_ctx* ctx, bool mixed);
int spmv_device(axia_ctx* ctx, bool fp32, const void* x, void* y, int lanes_req);
int bsr_autotune(axia_ctx* ctx, const char* cache_path, int* lanes_out, int* vec_out, double* us_out);
int batch_autotune(axia_ctx* ctx, const char* cache_path, int* tc_out, int* tu_out, double* us_out);
int64_t dofmap_n_full(const axia_dofmap* m);
int raw_system_from_triplets(axia_ctx* ctx, int64_t n, int64_t nt, const int64_t* h_i, const int64_t* h_j,
                             const double* h_v, bool fp32);
int raw_system_from_csr(axia_ctx* ctx, int64_t n, const int64_t* h_indptr, const int64_t* h_indices,
                        const double* h_data, bool fp32);

namespace {

struct EventTimer {
  cudaEvent_t a = nullptr, b = nullptr;
  cudaStream_t s;
  explicit EventTimer(cudaStream_t st) : s(st) {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, s);
  }
  double stop_ms() {
    cudaEventRecord(b, s);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
  }
  ~EventTimer() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
};

void free_mesh_state(axia_ctx* ctx) {
  // nothing of the old state may still be in use once its blocks are pooled
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  multimesh_release(ctx);
  coarse_release(ctx);
  ctx->mesh_node0.clear();
  ctx->mesh_blocks.clear();
  dev_release(ctx, ctx->d_coords);
  dev_release(ctx, ctx->d_conn);
  dev_release(ctx, ctx->d_e);
  dev_release(ctx, ctx->d_ind_of);
  dev_release(ctx, ctx->d_u0);
  dev_release(ctx, ctx->d_ne_ptr);
  dev_release(ctx, ctx->d_ne);
  dev_release(ctx, ctx->d_adj_ptr);
  dev_release(ctx, ctx->d_adj);
  dev_release(ctx, ctx->d_adj_off);
  dev_release(ctx, ctx->d_node_rowlen);
  dev_release(ctx, ctx->d_rowptr);
  dev_release(ctx, ctx->d_col);
  dev_release(ctx, ctx->d_val);
  dev_release(ctx, ctx->d_val32);
  dev_release(ctx, ctx->d_diag);
  dev_release(ctx, ctx->d_dinv);
  dev_release(ctx, ctx->d_dinv32);
  dev_release(ctx, ctx->d_kfu0);
  dev_release(ctx, ctx->d_ke);
  ctx->ke_elems = 0;
  dev_release(ctx, ctx->d_f);
  dev_release(ctx, ctx->d_u);
  dev_release(ctx, ctx->d_b);
  dev_release(ctx, ctx->d_x);
  dev_release(ctx, ctx->d_r);
  dev_release(ctx, ctx->d_p);
  dev_release(ctx, ctx->d_q);
  dev_release(ctx, ctx->d_b32);
  dev_release(ctx, ctx->d_x32);
  dev_release(ctx, ctx->d_r32);
  dev_release(ctx, ctx->d_p32);
  dev_release(ctx, ctx->d_q32);
  dev_release(ctx, ctx->d_adj_ptr32);
  dev_release(ctx, ctx->d_qptr);
  dev_release(ctx, ctx->d_qadj);
  ctx->nbq = 0;
  dev_release(ctx, ctx->d_bval64);
  dev_release(ctx, ctx->d_bval32);
  dev_release(ctx, ctx->d_bval32lo);
  ctx->have_bsr32lo = false;
  dev_release(ctx, ctx->d_uptr);
  dev_release(ctx, ctx->d_uval);
  dev_release(ctx, ctx->d_lptr);
  dev_release(ctx, ctx->d_low);
  ctx->nbu = ctx->nbl = 0;
  ctx->have_sym32 = false;
  dev_release(ctx, ctx->d_bdinv64);
  dev_release(ctx, ctx->d_bdinv32);
  dev_release(ctx, ctx->d_bf);
  dev_release(ctx, ctx->d_xf);
  dev_release(ctx, ctx->d_rf);
  dev_release(ctx, ctx->d_pf);
  dev_release(ctx, ctx->d_qf);
  dev_release(ctx, ctx->d_xf32);
  dev_release(ctx, ctx->d_rf32);
  dev_release(ctx, ctx->d_pf32);
  dev_release(ctx, ctx->d_qf32);
  dev_release(ctx, ctx->d_zf32);
  ctx->full_capacity = 0;
  dev_release(ctx, ctx->d_mB);
  dev_release(ctx, ctx->d_mX);
  dev_release(ctx, ctx->d_mX32);
  dev_release(ctx, ctx->d_mXh);
  dev_release(ctx, ctx->d_mXl);
  ctx->seg_capacity = 0;
  if (ctx->d_mstate) cudaFree(ctx->d_mstate);
  ctx->d_mstate = nullptr;
  dev_release(ctx, ctx->d_mR32);
  dev_release(ctx, ctx->d_mP32);
  dev_release(ctx, ctx->d_mQ32);
  dev_release(ctx, ctx->d_mZ32);
  dev_release(ctx, ctx->d_bpart);
  dev_release(ctx, ctx->d_bgram);
  dev_release(ctx, ctx->d_bsmall);
  ctx->bpart_capacity = 0;
  if (ctx->d_mout) cudaFree(ctx->d_mout);
  ctx->d_mout = nullptr;
  ctx->batch_capacity = 0;
  dev_release(ctx, ctx->d_rho);
  dev_release(ctx, ctx->d_energy);
  dev_release(ctx, ctx->d_grad);
  dev_release(ctx, ctx->d_rec);
  ctx->have_forward = false;
  ctx->vec_capacity = 0;
  ctx->assembled = ctx->have32 = ctx->have_csr64 = ctx->have_bsr64 = ctx->have_bsr32 = ctx->have_bsr32lo = false;
  ctx->n_free = ctx->nnz = 0;
}

int use_device(axia_ctx* ctx) {
  AXIA_CUDA(ctx, cudaSetDevice(ctx->device));
  ctx->last_error.clear();
  return AXIA_OK;
}

void fill_info_sizes(const axia_ctx* ctx, axia_solve_info* info) {
  info->n_free = ctx->n_free;
  info->nnz = ctx->nnz;
  info->ms_setup = ctx->ms_setup;
  info->ms_assemble = ctx->ms_assemble;
  info->bad_index = ctx->last_bad;
}

}  // namespace

extern "C" {

int32_t axia_gpu_abi_version(void) { return AXIA_GPU_ABI_VERSION; }

axia_ctx* axia_gpu_create(int32_t device, int32_t* status) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
    if (status) *status = AXIA_ERR_CUDA;
    return nullptr;
  }
  axia_ctx* ctx = new axia_ctx;
  ctx->device = device;
  int st = AXIA_OK;
  do {
    if (cudaSetDevice(device) != cudaSuccess) { st = AXIA_ERR_CUDA; break; }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) { st = AXIA_ERR_CUDA; break; }
    if (!prop.cooperativeLaunch) { st = AXIA_ERR_CUDA; break; }
    ctx->sm_count = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) != cudaSuccess) { st = AXIA_ERR_CUDA; break; }
    ctx->stream = ctx->own_stream;
    if (dev_alloc(ctx, &ctx->d_status, 1) != AXIA_OK) { st = AXIA_ERR_OOM; break; }
    if (ensure_pcg_state(ctx) != AXIA_OK) { st = AXIA_ERR_OOM; break; }
    if (reset_dev_status(ctx) != AXIA_OK) { st = AXIA_ERR_CUDA; break; }
  } while (0);
  if (st != AXIA_OK) {
    axia_gpu_destroy(ctx);
    if (status) *status = st;
    return nullptr;
  }
  if (status) *status = AXIA_OK;
  return ctx;
}

void axia_gpu_destroy(axia_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  free_mesh_state(ctx);
  dev_pool_clear(ctx);
  dev_free(ctx->d_partials);
  dev_free(ctx->d_totals);
  dev_free(ctx->d_bar);
  dev_free(ctx->d_first_bad);
  dev_free(ctx->d_status);
  if (ctx->d_out) cudaFree(ctx->d_out);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
}

const char* axia_gpu_last_error(const axia_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "no context"; }

int32_t axia_gpu_element_ke(axia_ctx* ctx, int32_t nn, int32_t reduced, int64_t n_elem, const double* xyz,
                            const double* e, double nu, double* ke, double* vol, int64_t* bad_elem) {
  if (!ctx) return AXIA_ERR_INVALID_ARG;
  AXIA_TRY(use_device(ctx));
  if (bad_elem) *bad_elem = -1;
  if ((nn != 4 && nn != 6 && nn != 8 && nn != 10 && nn != 15 && nn != 20) || n_elem < 0 ||
      (n_elem > 0 && (!xyz || !e || !ke)))
    return set_error(ctx, AXIA_ERR_INVALID_ARG, "element_ke: nn must be 4, 6, 8, 10, 15 or 20 and buffers non-null");
  if (nu >= 0.5 || nu <= -1.0 || !std::isfinite(nu))  // d_iso_3d, elem.rs:42-44
    return set_error(ctx, AXIA_ERR_MATERIAL, "invalid Poisson ratio nu=" + std::to_string(nu));
  if (n_elem == 0) return AXIA_OK;
  const int64_t kesz = 9LL * nn * nn;
  double *d_xyz = nullptr, *d_e = nullptr, *d_ke = nullptr, *d_vol = nullptr;
  int st = AXIA_OK;
  do {
    if ((st = dev_alloc(ctx, &d_xyz, (size_t)(n_elem * 3 * nn)))) break;
    if ((st = dev_alloc(ctx, &d_e, (size_t)n_elem))) break;
    if ((st = dev_alloc(ctx, &d_ke, (size_t)(n_elem * kesz)))) break;
    if ((st = dev_alloc(ctx, &d_vol, (size_t)n_elem))) break;
    cudaMemcpyAsync(d_xyz, xyz, n_elem * 3 * nn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(d_e, e, n_elem * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    if ((st = reset_dev_status(ctx))) break;
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
    a.status = ctx->d_status;
    if ((st = run_element_ke(ctx, nn, reduced, a))) break;
    if (cudaMemcpyAsync(ke, d_ke, n_elem * kesz * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess) {
      st = set_error(ctx, AXIA_ERR_CUDA, "copy of Ke");
      break;
    }
    if (vol) cudaMemcpyAsync(vol, d_vol, n_elem * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
      st = set_error(ctx, AXIA_ERR_CUDA, std::string("element_ke: ") + cudaGetErrorString(cudaGetLastError()));
      break;
    }
    DevStatus hs;
    if ((st = read_dev_status(ctx, &hs))) break;
    if (hs.first_error != ~0ull) {
      int code = (int)(hs.first_error & 0xff);
      if (bad_elem) *bad_elem = (int64_t)(hs.first_error >> 8);
      st = set_error(ctx, code, "element " + std::to_string(hs.first_error >> 8) + ": element_ke failed (code " +
                                    std::to_string(code) + ")");
    }
  } while (0);
  cudaStreamSynchronize(ctx->stream);  // (error paths) before the blocks return to the pool
  dev_release(ctx, d_xyz);
  dev_release(ctx, d_e);
  dev_release(ctx, d_ke);
  dev_release(ctx, d_vol);
  return st;
}

int32_t axia_gpu_setup(axia_ctx* ctx, const axia_mesh* mesh, int64_t n_bc, const int64_t* bc_dof,
                       const double* bc_val) {
  if (!ctx || !mesh) return AXIA_ERR_INVALID_ARG;
  AXIA_TRY(use_device(ctx));
  auto t0 = std::chrono::steady_clock::now();
  if ((mesh->nn != 4 && mesh->nn != 6 && mesh->nn != 8 && mesh->nn != 10 && mesh->nn != 15 && mesh->nn != 20) ||
      mesh->n_nodes <= 0 ||
      mesh->n_elem < 0 || !mesh->coords ||
      (mesh->n_elem > 0 && !mesh->conn) || n_bc < 0 || (n_bc > 0 && (!bc_dof || !bc_val)))
    return set_error(ctx, AXIA_ERR_INVALID_ARG, "setup: bad mesh description");
  if (mesh->n_elem >= (1LL << 26)) return set_error(ctx, AXIA_ERR_TOO_LARGE, "setup: more than 2^26 elements");
  if (3 * mesh->n_nodes >= (int64_t)INT32_MAX) return set_error(ctx, AXIA_ERR_TOO_LARGE, "setup: too many nodes");
  if (mesh->nu >= 0.5 || mesh->nu <= -1.0 || !std::isfinite(mesh->nu))
    return set_error(ctx, AXIA_ERR_MATERIAL, "invalid Poisson ratio nu=" + std::to_string(mesh->nu));
  if (!mesh->e_elem && !(mesh->e > 0.0))
    return set_error(ctx, AXIA_ERR_MATERIAL, "invalid Young's modulus E=" + std::to_string(mesh->e));
  free_mesh_state(ctx);
  ctx->nn = mesh->nn;
  // nn = 8: reduced 1 = C3D8R, 2 = C3D8I; nn = 20: reduced 1 = C3D20R
  ctx->reduced = mesh->nn == 20 ? (mesh->reduced ? 1 : 0)
                 : mesh->nn == 8 ? ((mesh->reduced == 1 || mesh->reduced == 2) ? mesh->reduced : 0)
                                 : 0;
  ctx->ngp = mesh->nn == 4 ? 1 : mesh->nn == 10 ? 4 : mesh->nn == 6 ? 6 : mesh->nn == 15 ? 9
             : (mesh->nn == 8 && ctx->reduced == 1) ? 1 : (mesh->nn == 8 || ctx->reduced) ? 8 : 27;
  ctx->n_nodes = mesh->n_nodes;
  ctx->n_elem = mesh->n_elem;
  ctx->nu = mesh->nu;
  ctx->ndof = 3 * mesh->n_nodes;
  ctx->last_bad = -1;
  const int64_t ndof = ctx->ndof;
  // prescribed DOFs, last BC wins (analysis.rs:556-565): checked here, mapped on the device
  for (int64_t k = 0; k < n_bc; ++k) {
    const int64_t d = bc_dof[k];
    if (d < 0 || d >= ndof) return set_error(ctx, AXIA_ERR_INVALID_ARG, "BC " + std::to_string(k) + " names DOF out of range");
    if (!std::isfinite(bc_val[k])) return set_error(ctx, AXIA_ERR_NONFINITE, "BC " + std::to_string(k) + " value not finite");
  }
  int64_t* d_bc_dof = nullptr;
  double* d_bc_val = nullptr;
  AXIA_TRY(dev_alloc(ctx, &d_bc_dof, (size_t)std::max<int64_t>(n_bc, 1)));
  AXIA_TRY(dev_alloc(ctx, &d_bc_val, (size_t)std::max<int64_t>(n_bc, 1)));
  if (n_bc > 0) {
    AXIA_CUDA(ctx, cudaMemcpyAsync(d_bc_dof, bc_dof, n_bc * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
    AXIA_CUDA(ctx, cudaMemcpyAsync(d_bc_val, bc_val, n_bc * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  }
  AXIA_TRY(dev_alloc(ctx, &ctx->d_coords, (size_t)(3 * mesh->n_nodes)));
  AXIA_TRY(dev_alloc(ctx, &ctx->d_conn, (size_t)(mesh->n_elem * mesh->nn)));
  AXIA_TRY(dev_alloc(ctx, &ctx->d_e, (size_t)std::max<int64_t>(mesh->n_elem, 1)));
  AXIA_CUDA(ctx, cudaMemcpyAsync(ctx->d_coords, mesh->coords, 3 * mesh->n_nodes * sizeof(double),
                                 cudaMemcpyHostToDevice, ctx->stream));
  if (mesh->n_elem > 0)
    AXIA_CUDA(ctx, cudaMemcpyAsync(ctx->d_conn, mesh->conn, mesh->n_elem * mesh->nn * sizeof(int32_t),
                                   cudaMemcpyHostToDevice, ctx->stream));
  if (mesh->e_elem) {
    AXIA_CUDA(ctx, cudaMemcpyAsync(ctx->d_e, mesh->e_elem, mesh->n_elem * sizeof(double), cudaMemcpyHostToDevice,
                                   ctx->stream));
  } else {
    std::vector<double> ev(std::max<int64_t>(mesh->n_elem, 1), mesh->e);
    AXIA_CUDA(ctx, cudaMemcpyAsync(ctx->d_e, ev.data(), ev.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  AXIA_TRY(reset_dev_status(ctx));
  int st = symbolic_setup(ctx, n_bc, d_bc_dof, d_bc_val);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  dev_release(ctx, d_bc_dof);
  dev_release(ctx, d_bc_val);
  if (st != AXIA_OK) return st;
  if (ctx->n_free == 0 && n_bc == 0)  // constraint.rs:111-113
    return set_error(ctx, AXIA_ERR_NO_FREE_DOF, "model without free degrees of freedom");
  ctx->ms_setup = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return AXIA_OK;
}

int32_t axia_gpu_assemble_ex(axia_ctx* ctx, int32_t flags) {
  if (!ctx) return AXIA_ERR_INVALID_ARG;
  AXIA_TRY(use_device(ctx));
  if (!ctx->d_rowptr || !ctx->d_conn) return set_error(ctx, AXIA_ERR_STATE, "assemble before setup");
  if (flags <= 0 || flags > 63) return set_error(ctx, AXIA_ERR_INVALID_ARG, "assemble: unknown matrix forms");
  if ((flags & AXIA_ASM_BSR32LO) && !(flags & AXIA_ASM_BSR32))
    return set_error(ctx, AXIA_ERR_INVALID_ARG, "assemble: AXIA_ASM_BSR32LO needs AXIA_ASM_BSR32");
  EventTimer t(ctx->stream);
  int st = numeric_assemble(ctx, flags);
  ctx->ms_assemble = t.stop_ms();
  return st;
}

int32_t axia_gpu_assemble(axia_ctx* ctx, int32_t precision) {
  return axia_gpu_assemble_ex(ctx, precision == AXIA_PREC_MIXED ? (AXIA_ASM_CSR64 | AXIA_ASM_CSR32) : AXIA_ASM_CSR64);
}

static int32_t solve_common(axia_ctx* ctx, const double* d_f, double* d_u, const axia_solve_opts* opts,
                            axia_solve_info* info) {
  axia_solve_info local{};
  if (!info) info = &local;
  std::memset(info, 0, sizeof(*info));
  info->bad_index = -1;
  axia_solve_opts o{};
  if (opts) {
    o = *opts;
  } else {
    o.rtol = 1e-8;
    o.precision = AXIA_PREC_FP64;
  }
  if (!(o.rtol > 0.0)) o.rtol = 1e-8;
  if (o.preconditioner != AXIA_PRECOND_JACOBI &&
      (o.preconditioner != AXIA_PRECOND_COARSE ||
       (o.matrix_format != AXIA_FORMAT_BSR3 && o.matrix_format != AXIA_FORMAT_BSR3_SYM) ||
       o.precision != AXIA_PREC_MIXED))
    return set_error(ctx, AXIA_ERR_INVALID_ARG, "the coarse preconditioner needs the mixed node-block solve");
  EventTimer t(ctx->stream);
  int st = AXIA_OK;
  if (ctx->n_free > 0 && (o.matrix_format == AXIA_FORMAT_BSR3 || o.matrix_format == AXIA_FORMAT_BSR3_SYM)) {
    st = bsr_solve(ctx, d_f, d_u, &o, info);
    info->ms_solve = t.stop_ms();
    fill_info_sizes(ctx, info);
    info->status = st;
    return st;
  }
  if (ctx->n_free > 0 && !ctx->have_csr64) st = set_error(ctx, AXIA_ERR_STATE, "CSR solve needs AXIA_ASM_CSR64");
  if (ctx->n_free > 0 && st == AXIA_OK) {
    st = prepare_solve(ctx, o.precision == AXIA_PREC_MIXED);
    if (st == AXIA_OK) st = build_rhs(ctx, d_f);
    if (st == AXIA_OK) st = pcg_solve(ctx, &o, info);
    if (st == AXIA_OK) st = reconstruct(ctx, d_u);
  } else {
    cudaMemcpyAsync(d_u, ctx->d_u0, ctx->ndof * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream);
  }
  info->ms_solve = t.stop_ms();
  if (st == AXIA_OK && ctx->n_free > 0) true_residual(ctx, &info->true_residual);
  fill_info_sizes(ctx, info);
  info->status = st;
  return st;
}

int32_t axia_gpu_solve_device(axia_ctx* ctx, const double* f_full_dev, double* u_full_dev,
                              const axia_solve_opts* opts, axia_solve_info* info) {
  if (!ctx || !f_full_dev || !u_full_dev) return AXIA_ERR_INVALID_ARG;
  AXIA_TRY(use_device(ctx));
  if (!ctx->assembled || !ctx->d_ind_of) return set_error(ctx, AXIA_ERR_STATE, "solve before assemble");
  return solve_common(ctx, f_full_dev, u_full_dev, opts, info);
}

int32_t axia_gpu_solve(axia_ctx* ctx, const double* f_full, double* u_full, const axia_solve_opts* opts,
                       axia_solve_info* info) {
  if (!ctx || !f_full || !u_full) return AXIA_ERR_INVALID_ARG;
  AXIA_TRY(use_device(ctx));
  if (!ctx->assembled || !ctx->d_ind_of) return set_error(ctx, AXIA_ERR_STATE, "solve before assemble");
  if (!ctx->d_f) AXIA_TRY(dev_alloc(ctx, &ctx->d_f, (size_t)ctx->ndof));
  if (!ctx->d_u) AXIA_TRY(dev_alloc(ctx, &ctx->d_u, (size_t)ctx->ndof));
  AXIA_CUDA(ctx, cudaMemcpyAsync(ctx->d_f, f_full, ctx->ndof * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  int64_t bad = -1;
  AXIA_TRY(device_first_nonfinite(ctx, ctx->d_f, ctx->ndof, &bad));
  if (bad >= 0) return set_error(ctx, AXIA_ERR_NONFINITE, "load vector entry " + std::to_string(bad) + " not finite");
  int st = solve_common(ctx, ctx->d_f, ctx->d_u, opts, info);
  if (st != AXIA_OK) return st;
  AXIA_CUDA(ctx, cudaMemcpyAsync(u_full, ctx->d_u, ctx->ndof * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return AXIA_OK;
}

// PCG on the context's raw K_ff (from triplets or CSR): rhs -> x, both host arrays.
static int32_t solve_raw(axia_ctx* ctx, const double* rhs, const double* d_rhs, double* x, const axia_solve_opts* opts,
                         axia_solve_info* info) {
  axia_solve_info local{};
  if (!info) info = &local;
  std::memset(info, 0, sizeof(*info));
  info->bad_index = -1;
  axia_solve_opts o{};
  if (opts) o = *opts;
  if (!(o.rtol > 0.0)) o.rtol = 1e-8;  // solve_kff's PCG tolerance (linalg.rs:363)
  if (o.matrix_format != AXIA_FORMAT_CSR || o.preconditioner != AXIA_PRECOND_JACOBI)
    return set_error(ctx, AXIA_ERR_INVALID_ARG,
                     "solve_kff: caller systems are CSR with Jacobi; node blocks and the coarse space need a mesh");
  const bool mixed = o.precision == AXIA_PREC_MIXED;
  EventTimer t(ctx->stream);
  int st = ensure_pcg_state(ctx);
  if (st == AXIA_OK) st = prepare_solve(ctx, mixed);
  if (st == AXIA_OK && cudaMemcpyAsync(ctx->d_b, d_rhs ? d_rhs : rhs, ctx->n_free * sizeof(double),
                                       d_rhs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                       ctx->stream) != cudaSuccess)
    st = set_error(ctx, AXIA_ERR_CUDA, "solve_kff: rhs upload");
  if (st == AXIA_OK) st = pcg_solve(ctx, &o, info);
  info->ms_solve = t.stop_ms();
  if (st == AXIA_OK) {
    true_residual(ctx, &info->true_residual);
    if (x && (cudaMemcpyAsync(x, ctx->d_x, ctx->n_free * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream) !=
                  cudaSuccess ||
              cudaStreamSynchronize(ctx->stream) != cudaSuccess))
      st = set_error(ctx, AXIA_ERR_CUDA, "solve_kff: solution download");
  }
  info->n_free = ctx->n_free;
  info->nnz = ctx->nnz;
  info->bad_index = ctx->last_bad;
  info->status = st;
  return st;
}

static int check_raw_rhs(axia_ctx* ctx, int64_t n, const double* rhs) {
  for (int64_t d = 0; d < n; ++d)
    if (!std::isfinite(rhs[d]))
      return set_error(ctx, AXIA_ERR_NONFINITE, "solve_kff: rhs entry " + std::to_string(d) + " not finite");
  return AXIA_OK;
}

int32_t axia_gpu_solve_triplets(axia_ctx* ctx, int64_t n, int64_t n_trips, const int64_t* ti, const int64_t* tj,
                                const double* tv, const double* rhs, double* x, const axia_solve_opts* opts,
                                axia_solve_info* info) {
  if (!ctx || !rhs || !x || n <= 0 || n_trips < 0 || (n_trips > 0 && (!ti || !tj || !tv)))
    return AXIA_ERR_INVALID_ARG;
  AXIA_TRY(use_device(ctx));
  AXIA_TRY(check_raw_rhs(ctx, n, rhs));
  free_mesh_state(ctx);
  const bool mixed = opts && opts->precision == AXIA_PREC_MIXED;
  AXIA_TRY(raw_system_from_triplets(ctx, n, n_trips, ti, tj, tv, mixed));
  return solve_raw(ctx, rhs, nullptr, x, opts, info);
}

int32_t axia_gpu_solve_reduced(axia_ctx* ctx, const axia_dofmap* map, int64_t n_trips, const int64_t* ti,
                               const int64_t* tj, const double* tv, const double* f_full, double* u_full,
                               const axia_solve_opts* opts, axia_solve_info* info) {
  if (!ctx || !map || !f_full || !u_full || n_trips < 0 || (n_trips > 0 && (!ti || !tj || !tv)))
    return AXIA_ERR_INVALID_ARG;
  AXIA_TRY(use_device(ctx));
  const int64_t nf = axia_dofmap_export(map, nullptr, nullptr, nullptr, nullptr, nullptr) >= 0 ? dofmap_n_full(map) : 0;
  AXIA_TRY(check_raw_rhs(ctx, nf, f_full));
  free_mesh_state(ctx);
  AXIA_TRY(reset_dev_status(ctx));
  const bool mixed = opts && opts->precision == AXIA_PREC_MIXED;
  ReducedSystem S;
  int st = reduce_system(ctx, map, n_trips, ti, tj, tv, f_full, mixed, &S);
  if (st == AXIA_OK && S.n_ind == 0) {  // everything prescribed or slaved: u = u0
    if (cudaMemcpyAsync(u_full, S.u0, nf * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
      st = set_error(ctx, AXIA_ERR_CUDA, "copy of u0");
    if (info) {
      std::memset(info, 0, sizeof(*info));
      info->bad_index = -1;
    }
    S.release();
    return st;
  }
  if (st == AXIA_OK) st = solve_raw(ctx, nullptr, S.rhs, nullptr, opts, info);
  double* du = nullptr;
  if (st == AXIA_OK) st = dev_alloc(ctx, &du, (size_t)nf);
  if (st == AXIA_OK) st = reconstruct_system(ctx, S, ctx->d_x, du);
  if (st == AXIA_OK && (cudaMemcpyAsync(u_full, du, nf * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream) !=
                            cudaSuccess ||
                        cudaStreamSynchronize(ctx->stream) != cudaSuccess))
    st = set_error(ctx, AXIA_ERR_CUDA, "copy of u");
  cudaStreamSynchronize(ctx->stream);
  dev_release(ctx, du);
  S.release();
  return st;
}

int32_t axia_gpu_solve_csr(axia_ctx* ctx, int64_t n, const int64_t* indptr, const int64_t* indices,
                           const double* data, const double* rhs, double* x, const axia_solve_opts* opts,
                           axia_solve_info* info) {
  if (!ctx || !indptr || !rhs || !x || n <= 0) return AXIA_ERR_INVALID_ARG;
  if (indptr[n] > 0 && (!indices || !data)) return AXIA_ERR_INVALID_ARG;
  AXIA_TRY(use_device(ctx));
  AXIA_TRY(check_raw_rhs(ctx, n, rhs));
  free_mesh_state(ctx);
  const bool mixed = opts && opts->precision == AXIA_PREC_MIXED;
  AXIA_TRY(raw_system_from_csr(ctx, n, indptr, indices, data, mixed));
  return solve_raw(ctx, rhs, nullptr, x, opts, info);
}

int32_t axia_gpu_autotune(axia_ctx* ctx, const char* cache_path, int32_t* lanes, int32_t* vec,
                          double* us_per_iter) {
  if (!ctx || !lanes || !vec) return AXIA_ERR_INVALID_ARG;
  AXIA_TRY(use_device(ctx));
  int l = 0, v = 0;
  AXIA_TRY(bsr_autotune(ctx, cache_path, &l, &v, us_per_iter));
  *lanes = l;
  *vec = v;
  return AXIA_OK;
}

int32_t axia_gpu_autotune_batched(axia_ctx* ctx, const char* cache_path, int32_t* cases_per_lane,
                                  int32_t* blocks_per_step, double* us_per_iter) {
  if (!ctx || !cases_per_lane || !blocks_per_step) return AXIA_ERR_INVALID_ARG;
  AXIA_TRY(use_device(ctx));
  int tc = 0, tu = 0;
  double us = 0.0;
  AXIA_TRY(batch_autotune(ctx, cache_path, &tc, &tu, &us));
  *cases_per_lane = tc;
  *blocks_per_step = tu;
  if (us_per_iter) *us_per_iter = us;
  return AXIA_OK;
}

int32_t axia_gpu_set_stream(axia_ctx* ctx, void* stream) {
  if (!ctx) return AXIA_ERR_INVALID_ARG;
  AXIA_TRY(use_device(ctx));
  AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
  return AXIA_OK;
}

int64_t axia_gpu_kernel_launches(const axia_ctx* ctx) { return ctx ? ctx->launches : -1; }

// One block at a barrier of two: the second arrival never comes, so the
// bounded wait runs out, records the timeout and returns.
__global__ void k_wait_probe(GridBarrier* bar, DevStatus* st, unsigned long long limit_ns) {
  (void)group_sync(bar, st, limit_ns, 2u);
}

int32_t axia_gpu_check_wait_limit(axia_ctx* ctx, int64_t limit_us, int32_t* status, double* elapsed_ms) {
  if (!ctx || !status || limit_us < 1 || limit_us > 10000000) return AXIA_ERR_INVALID_ARG;
  AXIA_TRY(use_device(ctx));
  if (!ctx->d_bar) AXIA_TRY(dev_alloc(ctx, &ctx->d_bar, 1));
  AXIA_TRY(reset_dev_status(ctx));
  AXIA_CUDA(ctx, cudaMemsetAsync(ctx->d_bar, 0, sizeof(GridBarrier), ctx->stream));
  cudaEvent_t a, b;
  AXIA_CUDA(ctx, cudaEventCreate(&a));
  AXIA_CUDA(ctx, cudaEventCreate(&b));
  cudaEventRecord(a, ctx->stream);
  k_wait_probe<<<1, 32, 0, ctx->stream>>>(ctx->d_bar, ctx->d_status, (unsigned long long)limit_us * 1000ull);
  ctx->launches++;
  cudaEventRecord(b, ctx->stream);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaEventSynchronize(b);
  float ms = 0.f;
  if (e == cudaSuccess) cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (e != cudaSuccess) return set_error(ctx, AXIA_ERR_CUDA, std::string("wait probe: ") + cudaGetErrorString(e));
  DevStatus hs;
  AXIA_TRY(read_dev_status(ctx, &hs));
  *status = hs.timeout ? AXIA_ERR_TIMEOUT : AXIA_OK;
  if (elapsed_ms) *elapsed_ms = ms;
  AXIA_CUDA(ctx, cudaMemsetAsync(ctx->d_bar, 0, sizeof(GridBarrier), ctx->stream));
  AXIA_TRY(reset_dev_status(ctx));
  AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return AXIA_OK;
}

int32_t axia_gpu_spmv_device(axia_ctx* ctx, int32_t precision, const void* x_dev, void* y_dev, int32_t lanes) {
  if (!ctx || !x_dev || !y_dev) return AXIA_ERR_INVALID_ARG;
  AXIA_TRY(use_device(ctx));
  if (!ctx->assembled) return set_error(ctx, AXIA_ERR_STATE, "spmv before assemble");
  const bool fp32 = precision == AXIA_PREC_MIXED;
  if (fp32 && !ctx->have32) return set_error(ctx, AXIA_ERR_STATE, "FP32 spmv needs axia_gpu_assemble(AXIA_PREC_MIXED)");
  if (!fp32 && !ctx->have_csr64) return set_error(ctx, AXIA_ERR_STATE, "FP64 spmv needs AXIA_ASM_CSR64");
  return spmv_device(ctx, fp32, x_dev, y_dev, lanes);
}

int32_t axia_gpu_bsr_spmv_device(axia_ctx* ctx, int32_t precision, const void* x_dev, void* y_dev, int32_t lanes,
                                 int32_t vec) {
  if (!ctx || !x_dev || !y_dev) return AXIA_ERR_INVALID_ARG;
  AXIA_TRY(use_device(ctx));
  if (!ctx->assembled) return set_error(ctx, AXIA_ERR_STATE, "spmv before assemble");
  return bsr_spmv_device(ctx, precision == AXIA_PREC_MIXED, x_dev, y_dev, lanes, vec);
}

int32_t axia_gpu_sym_spmv_device(axia_ctx* ctx, const float* x_dev, float* y_dev, int32_t lanes) {
  if (!ctx || !x_dev || !y_dev) return AXIA_ERR_INVALID_ARG;
  AXIA_TRY(use_device(ctx));
  if (!ctx->assembled) return set_error(ctx, AXIA_ERR_STATE, "spmv before assemble");
  return sym_spmv_device(ctx, x_dev, y_dev, lanes);
}

int64_t axia_gpu_sym_blocks(const axia_ctx* ctx, int64_t* lower_entries) {
  if (!ctx) return -1;
  if (lower_entries) *lower_entries = ctx->nbl;
  return ctx->nbu;
}

int64_t axia_gpu_node_blocks(const axia_ctx* ctx) { return ctx ? ctx->n_adj : -1; }

int32_t axia_gpu_assemble_times(const axia_ctx* ctx, double* ms_element, double* ms_gather) {
  if (!ctx || !ms_element || !ms_gather) return AXIA_ERR_INVALID_ARG;
  *ms_element = ctx->ms_element;
  *ms_gather = ctx->ms_gather;
  return AXIA_OK;
}

int32_t axia_gpu_set_element_arith(axia_ctx* ctx, int32_t arith) {
  if (!ctx) return AXIA_ERR_INVALID_ARG;
  if (arith != AXIA_ELEMENT_DWORD && arith != AXIA_ELEMENT_FP64)
    return set_error(ctx, AXIA_ERR_INVALID_ARG, "element arithmetic must be AXIA_ELEMENT_DWORD or AXIA_ELEMENT_FP64");
  ctx->element_fp64 = arith == AXIA_ELEMENT_FP64;
  return AXIA_OK;
}

int32_t axia_gpu_element_energy(axia_ctx* ctx, const double* u_full, const double* v_full, double* s) {
  if (!ctx || !u_full || !v_full || !s) return AXIA_ERR_INVALID_ARG;
  AXIA_TRY(use_device(ctx));
  if (!ctx->d_conn) return set_error(ctx, AXIA_ERR_STATE, "element energy before setup");
  double *du = nullptr, *dv = nullptr;
  AXIA_TRY(dev_alloc(ctx, &du, (size_t)ctx->ndof));
  int st = dev_alloc(ctx, &dv, (size_t)ctx->ndof);
  if (st == AXIA_OK && !ctx->d_energy) st = dev_alloc(ctx, &ctx->d_energy, (size_t)std::max<int64_t>(ctx->n_elem, 1));
  if (st == AXIA_OK) {
    cudaMemcpyAsync(du, u_full, ctx->ndof * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(dv, v_full, ctx->ndof * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    st = element_energy(ctx, du, dv, ctx->d_energy);
  }
  if (st == AXIA_OK && (cudaMemcpyAsync(s, ctx->d_energy, ctx->n_elem * sizeof(double), cudaMemcpyDeviceToHost,
                                       ctx->stream) != cudaSuccess ||
                        cudaStreamSynchronize(ctx->stream) != cudaSuccess))
    st = set_error(ctx, AXIA_ERR_CUDA, "copy of element energies");
  cudaStreamSynchronize(ctx->stream);
  dev_release(ctx, du);
  dev_release(ctx, dv);
  return st;
}

int32_t axia_gpu_compliance_forward(axia_ctx* ctx, const double* rho, double penal, double e0, const double* f_full,
                                    double* u_full, double* compliance, const axia_solve_opts* opts,
                                    axia_solve_info* info) {
  if (!ctx || !rho || !f_full || !u_full || !compliance) return AXIA_ERR_INVALID_ARG;
  AXIA_TRY(use_device(ctx));
  if (!ctx->d_rowptr || !ctx->d_conn) return set_error(ctx, AXIA_ERR_STATE, "compliance before setup");
  if (!(e0 > 0.0) || !std::isfinite(penal)) return set_error(ctx, AXIA_ERR_MATERIAL, "SIMP needs E0 > 0 and a finite p");
  ctx->have_forward = false;
  if (!ctx->d_rho) AXIA_TRY(dev_alloc(ctx, &ctx->d_rho, (size_t)std::max<int64_t>(ctx->n_elem, 1)));
  AXIA_CUDA(ctx, cudaMemcpyAsync(ctx->d_rho, rho, ctx->n_elem * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  AXIA_TRY(simp_modulus(ctx, ctx->d_rho, penal, e0));
  axia_solve_opts o{};
  if (opts) {
    o = *opts;
  } else {
    o.rtol = 1e-10;
  }
  const bool mixed = o.precision == AXIA_PREC_MIXED;
  int flags = o.matrix_format == AXIA_FORMAT_BSR3       ? (AXIA_ASM_BSR64 | (mixed ? AXIA_ASM_BSR32 : 0))
              : o.matrix_format == AXIA_FORMAT_BSR3_SYM ? (AXIA_ASM_BSR64 | AXIA_ASM_SYM32)
                                                        : (AXIA_ASM_CSR64 | (mixed ? AXIA_ASM_CSR32 : 0));
  AXIA_TRY(axia_gpu_assemble_ex(ctx, flags));
  AXIA_TRY(axia_gpu_solve(ctx, f_full, u_full, &o, info));
  AXIA_TRY(device_dot(ctx, ctx->d_f, ctx->d_u, ctx->ndof, compliance));
  ctx->simp_p = penal;
  ctx->simp_e0 = e0;
  ctx->have_forward = true;
  return AXIA_OK;
}

int32_t axia_gpu_compliance_backward(axia_ctx* ctx, double* grad) {
  if (!ctx || !grad) return AXIA_ERR_INVALID_ARG;
  AXIA_TRY(use_device(ctx));
  if (!ctx->have_forward) return set_error(ctx, AXIA_ERR_STATE, "compliance backward before forward");
  if (!ctx->d_energy) AXIA_TRY(dev_alloc(ctx, &ctx->d_energy, (size_t)std::max<int64_t>(ctx->n_elem, 1)));
  if (!ctx->d_grad) AXIA_TRY(dev_alloc(ctx, &ctx->d_grad, (size_t)std::max<int64_t>(ctx->n_elem, 1)));
  AXIA_TRY(element_energy(ctx, ctx->d_u, ctx->d_u, ctx->d_energy));
  AXIA_TRY(simp_gradient(ctx, ctx->d_rho, ctx->d_energy, ctx->simp_p, ctx->simp_e0, ctx->d_grad));
  AXIA_CUDA(ctx, cudaMemcpyAsync(grad, ctx->d_grad, ctx->n_elem * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return AXIA_OK;
}

static int32_t batched_common(axia_ctx* ctx, int32_t nrhs, const double* d_F, double* d_U,
                              const axia_solve_opts* opts, axia_solve_info* info, double* rel_res) {
  axia_solve_info local{};
  if (!info) info = &local;
  std::memset(info, 0, sizeof(*info));
  info->bad_index = -1;
  axia_solve_opts o{};
  if (opts) o = *opts;
  if (!(o.rtol > 0.0)) o.rtol = 1e-8;
  EventTimer t(ctx->stream);
  int st = o.krylov == AXIA_KRYLOV_BLOCK ? batch_block_solve(ctx, nrhs, d_F, d_U, &o, info, rel_res)
                                        : batch_solve(ctx, nrhs, d_F, d_U, &o, info, rel_res);
  info->ms_solve = t.stop_ms();
  fill_info_sizes(ctx, info);
  info->status = st;
  return st;
}

int32_t axia_gpu_solve_batched_device(axia_ctx* ctx, int32_t nrhs, const double* F_dev, double* U_dev,
                                      const axia_solve_opts* opts, axia_solve_info* info, double* rel_res) {
  if (!ctx || nrhs < 0 || (nrhs > 0 && (!F_dev || !U_dev))) return AXIA_ERR_INVALID_ARG;
  AXIA_TRY(use_device(ctx));
  if (!ctx->assembled) return set_error(ctx, AXIA_ERR_STATE, "batched solve before assemble");
  if (nrhs == 0) return AXIA_OK;
  return batched_common(ctx, nrhs, F_dev, U_dev, opts, info, rel_res);
}

int32_t axia_gpu_solve_batched(axia_ctx* ctx, int32_t nrhs, const double* F, double* U, const axia_solve_opts* opts,
                               axia_solve_info* info, double* rel_res) {
  if (!ctx || nrhs < 0 || (nrhs > 0 && (!F || !U))) return AXIA_ERR_INVALID_ARG;
  AXIA_TRY(use_device(ctx));
  if (!ctx->assembled) return set_error(ctx, AXIA_ERR_STATE, "batched solve before assemble");
  if (nrhs == 0) return AXIA_OK;
  const size_t count = (size_t)nrhs * (size_t)ctx->ndof;
  double *dF = nullptr, *dU = nullptr;
  AXIA_TRY(dev_alloc(ctx, &dF, count));
  int st = dev_alloc(ctx, &dU, count);
  if (st == AXIA_OK &&
      cudaMemcpyAsync(dF, F, count * sizeof(double), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
    st = set_error(ctx, AXIA_ERR_CUDA, "copy of the load cases");
  if (st == AXIA_OK) {
    int64_t bad = -1;
    st = device_first_nonfinite(ctx, dF, (int64_t)count, &bad);
    if (st == AXIA_OK && bad >= 0) st = set_error(ctx, AXIA_ERR_NONFINITE, "load case entry not finite");
  }
  if (st == AXIA_OK) st = batched_common(ctx, nrhs, dF, dU, opts, info, rel_res);
  if (st == AXIA_OK) {
    if (cudaMemcpyAsync(U, dU, count * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
      st = set_error(ctx, AXIA_ERR_CUDA, "copy of batched solutions");
  }
  cudaStreamSynchronize(ctx->stream);
  dev_release(ctx, dF);
  dev_release(ctx, dU);
  return st;
}

int32_t axia_gpu_system_size(const axia_ctx* ctx, int64_t* n_free, int64_t* nnz) {
  if (!ctx) return AXIA_ERR_INVALID_ARG;
  if (n_free) *n_free = ctx->n_free;
  if (nnz) *nnz = ctx->nnz;
  return AXIA_OK;
}

int32_t axia_gpu_export_system(const axia_ctx* ctx_c, int32_t* rowptr, int32_t* col, double* val, double* diag,
                               double* kfu0) {
  axia_ctx* ctx = const_cast<axia_ctx*>(ctx_c);
  if (!ctx) return AXIA_ERR_INVALID_ARG;
  AXIA_TRY(use_device(ctx));
  if (!ctx->d_rowptr) return set_error(ctx, AXIA_ERR_STATE, "export before setup");
  AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // the copies below run on the legacy stream
  const int64_t n = ctx->n_free, nnz = ctx->nnz;
  if (rowptr) AXIA_CUDA(ctx, cudaMemcpy(rowptr, ctx->d_rowptr, (n + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost));
  if (col) {
    AXIA_TRY(ensure_csr_columns(ctx));
    AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    AXIA_CUDA(ctx, cudaMemcpy(col, ctx->d_col, nnz * sizeof(int32_t), cudaMemcpyDeviceToHost));
  }
  if ((val || diag || kfu0) && !ctx->assembled) return set_error(ctx, AXIA_ERR_STATE, "export of values before assemble");
  if (val && !ctx->have_csr64) return set_error(ctx, AXIA_ERR_STATE, "export of CSR values needs AXIA_ASM_CSR64");
  if (val) AXIA_CUDA(ctx, cudaMemcpy(val, ctx->d_val, nnz * sizeof(double), cudaMemcpyDeviceToHost));
  if (diag) AXIA_CUDA(ctx, cudaMemcpy(diag, ctx->d_diag, n * sizeof(double), cudaMemcpyDeviceToHost));
  if (kfu0 && ctx->d_kfu0) AXIA_CUDA(ctx, cudaMemcpy(kfu0, ctx->d_kfu0, n * sizeof(double), cudaMemcpyDeviceToHost));
  if (kfu0 && !ctx->d_kfu0) std::memset(kfu0, 0, n * sizeof(double));
  return AXIA_OK;
}

int32_t axia_gpu_export_dofmap(const axia_ctx* ctx_c, int32_t* ind_of) {
  axia_ctx* ctx = const_cast<axia_ctx*>(ctx_c);
  if (!ctx || !ind_of) return AXIA_ERR_INVALID_ARG;
  if (!ctx->d_ind_of) return AXIA_ERR_STATE;
  AXIA_TRY(use_device(ctx));
  AXIA_CUDA(ctx, cudaMemcpyAsync(ind_of, ctx->d_ind_of, ctx->ndof * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                 ctx->stream));
  AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return AXIA_OK;
}

}  // extern "C"
