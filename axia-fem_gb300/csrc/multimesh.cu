// multimesh.cu -- many independent meshes (e.g. a family of cubes of uneven
// size) set up and solved together.
//
// axia_gpu_setup_multi concatenates the meshes (node and element ids offset
// per mesh) into one context, so the symbolic phase and the assembly run once
// over all of them; the node-block matrix is then block diagonal with one
// diagonal block per mesh.  axia_gpu_solve_multi gives every mesh its own
// group of co-resident blocks -- at least one, more in proportion to its
// estimated work (node blocks x nodes^(1/3), the growth of CG iteration
// counts with mesh size) -- and runs all groups in one cooperative launch of
// pcg_group_reliable_kernel: each group runs the mixed-precision CG of its
// own mesh (FP32 node-block CG with FP64 reliable updates) with its own
// barrier and convergence test, and leaves when its mesh has converged.  The
// sequence (right-hand side, barrier reset, persistent solve, reconstruct) is
// captured once into a CUDA graph and replayed; the graph is rebuilt when the
// device buffers or options change.
//
// The reference solves each model separately (one solve_kff per model,
// solver/src/linalg.rs:311); the per-mesh recurrence is its pcg
// (linalg.rs:199-259).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "coarse.cuh"

extern "C" int32_t axia_gpu_setup(axia_ctx* ctx, const axia_mesh* mesh, int64_t n_bc, const int64_t* bc_dof,
                                  const double* bc_val);

namespace {

void drop_graph(axia_ctx* ctx) {
  if (ctx->multi_graph) cudaGraphExecDestroy((cudaGraphExec_t)ctx->multi_graph);
  ctx->multi_graph = nullptr;
}

int plan_groups(axia_ctx* ctx, int lanes, int vec, bool coarse) {
  const int nm = (int)ctx->mesh_node0.size() - 1;
  int per_sm = 0;
  AXIA_TRY(group_kernel_capacity(ctx, lanes, vec, &per_sm, coarse));
  const int cap = std::max(1, per_sm) * ctx->sm_count;
  if (nm > cap)
    return set_error(ctx, AXIA_ERR_TOO_LARGE, std::to_string(nm) + " meshes exceed the " + std::to_string(cap) +
                                                  " co-resident blocks of one launch");
  std::vector<double> w(nm);
  double wsum = 0.0;
  for (int k = 0; k < nm; ++k) {
    const double nodes = (double)(ctx->mesh_node0[k + 1] - ctx->mesh_node0[k]);
    w[k] = std::max(1.0, (double)ctx->mesh_blocks[k]) * std::max(1.0, std::cbrt(nodes));
    wsum += w[k];
  }
  // blocks in proportion to the work, at least one each; the blocks left by
  // rounding down go to the groups with the largest remainders
  std::vector<int> nc(nm);
  std::vector<double> rem(nm);
  int total = 0;
  for (int k = 0; k < nm; ++k) {
    const double share = cap * w[k] / wsum;
    nc[k] = std::max(1, (int)std::floor(share));
    rem[k] = share - std::floor(share);
    total += nc[k];
  }
  while (total > cap) {  // trim the largest groups
    int big = (int)(std::max_element(nc.begin(), nc.end()) - nc.begin());
    --nc[big];
    --total;
  }
  while (total < cap) {
    int k = (int)(std::max_element(rem.begin(), rem.end()) - rem.begin());
    if (rem[k] <= 0.0) break;
    ++nc[k];
    rem[k] = 0.0;
    ++total;
  }
  std::vector<MeshGroup> groups(nm);
  std::vector<int> cta_group(total);
  long long part = 0;
  int cta = 0;
  for (int k = 0; k < nm; ++k) {
    groups[k] = MeshGroup{(int)ctx->mesh_node0[k], (int)ctx->mesh_node0[k + 1], cta, nc[k], part, 0, 0, 0, 0};
    for (int j = 0; j < nc[k]; ++j) cta_group[cta + j] = k;
    cta += nc[k];
    part += (long long)GROUP_SLOTS * nc[k];
  }
  if ((size_t)part > ctx->partial_slots) return set_error(ctx, AXIA_ERR_TOO_LARGE, "partials area too small");
  AXIA_TRY(dev_alloc(ctx, &ctx->d_mgroups, sizeof(MeshGroup) * nm));
  AXIA_TRY(dev_alloc(ctx, &ctx->d_mcta, (size_t)total));
  AXIA_TRY(dev_alloc(ctx, &ctx->d_mbars, (size_t)nm));
  AXIA_TRY(dev_alloc(ctx, &ctx->d_mtotals, (size_t)4 * nm));
  AXIA_TRY(dev_alloc(ctx, &ctx->d_mouts, sizeof(PcgOut) * nm));
  AXIA_CUDA(ctx, cudaMemcpy(ctx->d_mgroups, groups.data(), sizeof(MeshGroup) * nm, cudaMemcpyHostToDevice));
  AXIA_CUDA(ctx, cudaMemcpy(ctx->d_mcta, cta_group.data(), sizeof(int) * total, cudaMemcpyHostToDevice));
  ctx->multi_grid = total;
  ctx->multi_lanes = lanes;
  ctx->multi_vec = vec;
  ctx->multi_coarse = coarse;
  ctx->multi_ctas.assign(nc.begin(), nc.end());
  drop_graph(ctx);
  return AXIA_OK;
}

int capture_graph(axia_ctx* ctx, const double* d_f, double* d_u, double rtol, double delta, long long max_iter,
                  const CoarseArgs* coarse) {
  drop_graph(ctx);
  BsrReliableArgs args = make_reliable_args(ctx, rtol, delta, max_iter);
  if (coarse) args.C = *coarse;
  const int64_t launches_before = ctx->launches;  // captured launches are counted when the graph runs
  cudaGraph_t g = nullptr;
  AXIA_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  int rc = launch_full_rhs(ctx, d_f);
  if (rc == AXIA_OK && cudaMemsetAsync(ctx->d_mbars, 0, sizeof(GridBarrier) * (ctx->mesh_node0.size() - 1),
                                       ctx->stream) != cudaSuccess)
    rc = set_error(ctx, AXIA_ERR_CUDA, "barrier reset in capture");
  if (rc == AXIA_OK)
    rc = launch_group_reliable(ctx, args, (const MeshGroup*)ctx->d_mgroups,
                               ctx->d_mcta, ctx->d_mbars, ctx->d_mtotals, (PcgOut*)ctx->d_mouts, ctx->multi_grid,
                               ctx->multi_lanes, ctx->multi_vec, coarse != nullptr);
  if (rc == AXIA_OK) rc = launch_full_reconstruct(ctx, d_u);
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  ctx->launches = launches_before;
  if (rc != AXIA_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return set_error(ctx, AXIA_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  cudaGraphExec_t ex = nullptr;
  e = cudaGraphInstantiate(&ex, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return set_error(ctx, AXIA_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  ctx->multi_graph = ex;
  ctx->graph_f = d_f;
  ctx->graph_u = d_u;
  ctx->graph_rtol = rtol;
  ctx->graph_delta = delta;
  ctx->graph_max_iter = max_iter;
  ctx->graph_coarse = coarse ? ctx->coarse_gen : -1;
  return AXIA_OK;
}

// the restriction chunks, coarse rows and block of the coarse inverse of every group
int set_group_ranges(axia_ctx* ctx) {
  const int nm = (int)ctx->mesh_node0.size() - 1;
  std::vector<int> c0, c1, r0, r1, col0, ldm;
  std::vector<long long> moff;
  AXIA_TRY(coarse_mesh_ranges(ctx, c0, c1, r0, r1, col0, ldm, moff));
  if ((int)c0.size() != nm) return set_error(ctx, AXIA_ERR_STATE, "coarse space does not match the meshes");
  std::vector<MeshGroup> g(nm);
  AXIA_CUDA(ctx, cudaMemcpyAsync(g.data(), ctx->d_mgroups, sizeof(MeshGroup) * nm, cudaMemcpyDeviceToHost,
                                 ctx->stream));
  AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  for (int k = 0; k < nm; ++k) {
    g[k].chunk0 = c0[k];
    g[k].chunk1 = c1[k];
    g[k].row0 = r0[k];
    g[k].row1 = r1[k];
    g[k].col0 = col0[k];
    g[k].ldm = ldm[k];
    g[k].moff = moff[k];
  }
  AXIA_CUDA(ctx, cudaMemcpyAsync(ctx->d_mgroups, g.data(), sizeof(MeshGroup) * nm, cudaMemcpyHostToDevice,
                                 ctx->stream));
  AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return AXIA_OK;
}

int solve_multi_device(axia_ctx* ctx, const double* d_f, double* d_u, const axia_solve_opts* opts,
                       axia_solve_info* info, double* rel_res, int64_t* iters) {
  if (ctx->mesh_node0.size() < 2) return set_error(ctx, AXIA_ERR_STATE, "solve_multi needs axia_gpu_setup_multi");
  if (!ctx->have_bsr64 || !ctx->have_bsr32)
    return set_error(ctx, AXIA_ERR_STATE, "solve_multi needs axia_gpu_assemble_ex(AXIA_ASM_BSR64 | AXIA_ASM_BSR32)");
  if (opts->preconditioner != AXIA_PRECOND_JACOBI && opts->preconditioner != AXIA_PRECOND_COARSE)
    return set_error(ctx, AXIA_ERR_INVALID_ARG, "solve_multi: unknown preconditioner");
  const bool coarse = opts->preconditioner == AXIA_PRECOND_COARSE;
  const int nm = (int)ctx->mesh_node0.size() - 1;
  AXIA_TRY(prepare_full_buffers(ctx));
  int lanes = 0, vec = 0;
  group_layout(ctx, opts->spmv_lanes, opts->spmv_vec, &lanes, &vec);
  if (ctx->multi_grid == 0 || ctx->multi_lanes != lanes || ctx->multi_vec != vec || ctx->multi_coarse != coarse)
    AXIA_TRY(plan_groups(ctx, lanes, vec, coarse));
  CoarseArgs cargs{};
  if (coarse) {  // per-mesh subdomains; the operator follows every assembly (outside the graph)
    AXIA_TRY(coarse_prepare(ctx, opts->coarse_nodes, &cargs, true));
    AXIA_TRY(set_group_ranges(ctx));
  }
  const double delta = opts->inner_rtol > 0 && opts->inner_rtol < 1 ? opts->inner_rtol : 0.01;
  long long max_iter = opts->max_iter > 0 ? opts->max_iter : 0;
  if (max_iter == 0) {
    int64_t biggest = 0;
    for (int k = 0; k < nm; ++k) biggest = std::max<int64_t>(biggest, 3 * (ctx->mesh_node0[k + 1] - ctx->mesh_node0[k]));
    max_iter = std::max<long long>(4 * biggest, 200);
  }
  // the space's generation, not an address: a rebuilt space may reuse some
  // released blocks of the pool and not others
  const int64_t coarse_key = coarse ? ctx->coarse_gen : -1;
  if (!ctx->multi_graph || ctx->graph_f != d_f || ctx->graph_u != d_u || ctx->graph_rtol != opts->rtol ||
      ctx->graph_delta != delta || ctx->graph_max_iter != max_iter || ctx->graph_coarse != coarse_key)
    AXIA_TRY(capture_graph(ctx, d_f, d_u, opts->rtol, delta, max_iter, coarse ? &cargs : nullptr));
  AXIA_TRY(reset_dev_status(ctx));
  cudaEvent_t a, b;
  AXIA_CUDA(ctx, cudaEventCreate(&a));
  AXIA_CUDA(ctx, cudaEventCreate(&b));
  cudaEventRecord(a, ctx->stream);
  cudaError_t e = cudaGraphLaunch((cudaGraphExec_t)ctx->multi_graph, ctx->stream);
  cudaEventRecord(b, ctx->stream);
  cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (e != cudaSuccess) return set_error(ctx, AXIA_ERR_CUDA, std::string("graph launch: ") + cudaGetErrorString(e));
  ctx->launches += 3;  // rhs, persistent solve, reconstruct
  info->ms_pcg_kernel = ms;
  info->pcg_launches = 1;
  std::vector<PcgOut> outs(nm);
  AXIA_CUDA(ctx, cudaMemcpyAsync(outs.data(), ctx->d_mouts, sizeof(PcgOut) * nm, cudaMemcpyDeviceToHost, ctx->stream));
  AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  DevStatus hs;
  AXIA_TRY(read_dev_status(ctx, &hs));
  if (hs.timeout) return set_error(ctx, AXIA_ERR_TIMEOUT, "a group barrier of the multi-mesh solve ran past its limit");
  int64_t it_max = 0, upd = 0;
  double worst = 0.0;
  int status = AXIA_OK, bad = -1;
  for (int k = 0; k < nm; ++k) {
    it_max = std::max<int64_t>(it_max, outs[k].iters);
    upd += outs[k].updates;
    const double rr = outs[k].bnorm > 0 ? outs[k].residual / outs[k].bnorm : 0.0;
    worst = std::max(worst, rr);
    if (rel_res) rel_res[k] = rr;
    if (iters) iters[k] = outs[k].iters;
    if (outs[k].status != AXIA_OK && status == AXIA_OK) {
      status = outs[k].status;
      bad = k;
    }
  }
  info->iters = it_max;
  info->outer_iters = upd;
  info->residual = worst;
  info->bnorm = 1.0;
  if (status != AXIA_OK) {
    info->bad_index = bad;
    return set_error(ctx, status, "mesh " + std::to_string(bad) + ": CG failed (status " + std::to_string(status) + ")");
  }
  return AXIA_OK;
}

}  // namespace

void multimesh_release(axia_ctx* ctx) {
  drop_graph(ctx);
  dev_free(ctx->d_mgroups);
  dev_free(ctx->d_mcta);
  dev_free(ctx->d_mbars);
  dev_free(ctx->d_mtotals);
  dev_free(ctx->d_mouts);
  ctx->multi_grid = 0;
  ctx->multi_lanes = 0;
  ctx->multi_vec = 0;
  ctx->multi_ctas.clear();
}

extern "C" {

int32_t axia_gpu_setup_multi(axia_ctx* ctx, int32_t n_meshes, const axia_mesh* meshes, const int64_t* n_bc,
                             const int64_t* const* bc_dof, const double* const* bc_val) {
  if (!ctx || n_meshes <= 0 || !meshes || !n_bc || !bc_dof || !bc_val) return AXIA_ERR_INVALID_ARG;
  const axia_mesh& m0 = meshes[0];
  int64_t nodes = 0, elems = 0, bcs = 0;
  for (int k = 0; k < n_meshes; ++k) {
    const axia_mesh& m = meshes[k];
    if (m.nn != m0.nn || (m.reduced != 0) != (m0.reduced != 0) || m.nu != m0.nu)
      return set_error(ctx, AXIA_ERR_INVALID_ARG, "setup_multi: all meshes need the same element type and nu");
    if (m.n_nodes <= 0 || m.n_elem < 0 || !m.coords || (m.n_elem > 0 && !m.conn) || n_bc[k] < 0 ||
        (n_bc[k] > 0 && (!bc_dof[k] || !bc_val[k])))
      return set_error(ctx, AXIA_ERR_INVALID_ARG, "setup_multi: bad mesh " + std::to_string(k));
    nodes += m.n_nodes;
    elems += m.n_elem;
    bcs += n_bc[k];
  }
  std::vector<double> coords(3 * nodes), e(std::max<int64_t>(elems, 1));
  std::vector<int32_t> conn((size_t)elems * m0.nn);
  std::vector<int64_t> bd(bcs);
  std::vector<double> bv(bcs);
  std::vector<int64_t> node0(n_meshes + 1, 0), elem0(n_meshes + 1, 0);
  int64_t no = 0, eo = 0, bo = 0;
  for (int k = 0; k < n_meshes; ++k) {
    const axia_mesh& m = meshes[k];
    node0[k] = no;
    elem0[k] = eo;
    std::memcpy(coords.data() + 3 * no, m.coords, sizeof(double) * 3 * m.n_nodes);
    for (int64_t i = 0; i < m.n_elem * m.nn; ++i) {
      const int32_t v = m.conn[i];
      if (v < 0 || v >= m.n_nodes)
        return set_error(ctx, AXIA_ERR_INVALID_ARG, "setup_multi: mesh " + std::to_string(k) + " names a node out of range");
      conn[(size_t)eo * m0.nn + i] = (int32_t)(v + no);
    }
    for (int64_t i = 0; i < m.n_elem; ++i) e[eo + i] = m.e_elem ? m.e_elem[i] : m.e;
    for (int64_t i = 0; i < n_bc[k]; ++i) {
      if (bc_dof[k][i] < 0 || bc_dof[k][i] >= 3 * m.n_nodes)
        return set_error(ctx, AXIA_ERR_INVALID_ARG, "setup_multi: mesh " + std::to_string(k) + " BC out of range");
      bd[bo + i] = bc_dof[k][i] + 3 * no;
      bv[bo + i] = bc_val[k][i];
    }
    no += m.n_nodes;
    eo += m.n_elem;
    bo += n_bc[k];
  }
  node0[n_meshes] = no;
  elem0[n_meshes] = eo;
  if (no >= (int64_t)INT32_MAX / 3) return set_error(ctx, AXIA_ERR_TOO_LARGE, "setup_multi: too many nodes");
  axia_mesh u = m0;
  u.n_nodes = nodes;
  u.coords = coords.data();
  u.n_elem = elems;
  u.conn = conn.data();
  u.e_elem = e.data();
  multimesh_release(ctx);
  ctx->mesh_node0.clear();
  int32_t st = axia_gpu_setup(ctx, &u, bcs, bd.data(), bv.data());
  if (st != AXIA_OK) return st;
  // node blocks per mesh, from the block-row pointers
  std::vector<int64_t> adj_ptr(nodes + 1);
  AXIA_CUDA(ctx, cudaMemcpy(adj_ptr.data(), ctx->d_adj_ptr, sizeof(int64_t) * (nodes + 1), cudaMemcpyDeviceToHost));
  ctx->mesh_blocks.assign(n_meshes, 0);
  for (int k = 0; k < n_meshes; ++k) ctx->mesh_blocks[k] = adj_ptr[node0[k + 1]] - adj_ptr[node0[k]];
  ctx->mesh_node0 = node0;
  return AXIA_OK;
}

int32_t axia_gpu_solve_multi_device(axia_ctx* ctx, const double* f_full_dev, double* u_full_dev,
                                    const axia_solve_opts* opts, axia_solve_info* info, double* rel_res,
                                    int64_t* iters) {
  if (!ctx || !f_full_dev || !u_full_dev) return AXIA_ERR_INVALID_ARG;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return AXIA_ERR_CUDA;
  ctx->last_error.clear();
  axia_solve_info local{};
  if (!info) info = &local;
  std::memset(info, 0, sizeof(*info));
  info->bad_index = -1;
  axia_solve_opts o{};
  if (opts) o = *opts;
  if (!(o.rtol > 0.0)) o.rtol = 1e-8;
  const int st = solve_multi_device(ctx, f_full_dev, u_full_dev, &o, info, rel_res, iters);
  info->ms_solve = info->ms_pcg_kernel;
  info->n_free = ctx->n_free;
  info->nnz = ctx->nnz;
  info->ms_setup = ctx->ms_setup;
  info->ms_assemble = ctx->ms_assemble;
  info->status = st;
  return st;
}

int32_t axia_gpu_solve_multi(axia_ctx* ctx, const double* f_full, double* u_full, const axia_solve_opts* opts,
                             axia_solve_info* info, double* rel_res, int64_t* iters) {
  if (!ctx || !f_full || !u_full) return AXIA_ERR_INVALID_ARG;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return AXIA_ERR_CUDA;
  for (int64_t d = 0; d < ctx->ndof; ++d)
    if (!std::isfinite(f_full[d])) return set_error(ctx, AXIA_ERR_NONFINITE, "load vector entry not finite");
  if (!ctx->d_f) AXIA_TRY(dev_alloc(ctx, &ctx->d_f, (size_t)ctx->ndof));
  if (!ctx->d_u) AXIA_TRY(dev_alloc(ctx, &ctx->d_u, (size_t)ctx->ndof));
  AXIA_CUDA(ctx, cudaMemcpyAsync(ctx->d_f, f_full, ctx->ndof * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  const int st = axia_gpu_solve_multi_device(ctx, ctx->d_f, ctx->d_u, opts, info, rel_res, iters);
  if (st != AXIA_OK) return st;
  AXIA_CUDA(ctx, cudaMemcpyAsync(u_full, ctx->d_u, ctx->ndof * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  AXIA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return AXIA_OK;
}

}  // extern "C"
