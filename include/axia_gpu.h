/*
 * axia_gpu.h -- C ABI of the GB300 (sm_103a) linear-static backend for Axia.
 *
 * The library replaces, for C3D8 / C3D20(R) continuum models with isotropic
 * material and single-point constraints, the *STATIC hot path of the
 * reference solver crate (larsmei/axia-fem, crate axia-fem 1.31.10):
 *
 *   element_ke            solver/src/elem.rs:344-375 (Hex8 arm),
 *                         solver/src/elem.rs:487-495 (Hex20/Hex20R arm)
 *   element loop + triplet push   solver/src/analysis.rs:574-668
 *   DofMap::build/reduce  solver/src/constraint.rs:26-172 (prescribed subset)
 *   solve_kff             solver/src/linalg.rs:311-404 (csr_from_triplets
 *                         linalg.rs:10-38, pcg linalg.rs:199-259)
 *   DofMap::reconstruct   solver/src/constraint.rs:207-217
 *
 * All pointers are host pointers unless the function name ends in _device.
 * The caller owns every buffer; the library copies what it needs into device
 * memory held by the context.  Every call is synchronous: it returns after
 * the device work has finished.  Errors are status codes, never aborts; the
 * message of the last error is available from axia_gpu_last_error().
 *
 * Threading: a context belongs to one host thread at a time (the reference
 * selects its backend per process or per thread, solver/src/backend.rs:49-89).
 */
#ifndef AXIA_GPU_H
#define AXIA_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AXIA_GPU_ABI_VERSION 2

#if defined(__GNUC__)
#define AXIA_API __attribute__((visibility("default")))
#else
#define AXIA_API
#endif

/* Status codes.  The reference returns Result<_, FemError(String)>
 * (solver/src/error.rs:1-18); each code names the reference error it stands for. */
typedef enum axia_status {
  AXIA_OK = 0,
  AXIA_ERR_INVALID_ARG = 1,        /* bad size, index or pointer */
  AXIA_ERR_SINGULAR_JACOBIAN = 2,  /* |det J| < 1e-18, elem.rs:14-16 */
  AXIA_ERR_NEG_JACOBIAN = 3,       /* det J <= 0, elem.rs:208-210, quadratic.rs:137-139 */
  AXIA_ERR_MATERIAL = 4,           /* nu >= 0.5, nu <= -1 or E <= 0, elem.rs:42-47 */
  AXIA_ERR_NOT_CONVERGED = 5,      /* final ||r|| > 10 tol ||b||, linalg.rs:253-257 */
  AXIA_ERR_ZERO_PIVOT = 6,         /* |p.Ap| < 1e-30, linalg.rs:231-232 */
  AXIA_ERR_NO_FREE_DOF = 9,        /* constraint.rs:111-113 */
  AXIA_ERR_NONFINITE = 10,         /* NaN / Inf in coordinates, loads or iterates */
  AXIA_ERR_CUDA = 11,              /* a CUDA runtime call failed */
  AXIA_ERR_OOM = 12,               /* device allocation failed */
  AXIA_ERR_TIMEOUT = 13,           /* a device-side wait ran past its limit */
  AXIA_ERR_STATE = 14,             /* call order: e.g. solve before setup */
  AXIA_ERR_TOO_LARGE = 15          /* a size above a documented limit */
} axia_status;

typedef enum axia_precision {
  AXIA_PREC_FP64 = 0,   /* K in FP64 CSR, FP64 Jacobi-PCG */
  AXIA_PREC_MIXED = 1   /* K in FP32 CSR for an FP32 inner PCG, FP64 residual and update */
} axia_precision;

/* Matrix forms axia_gpu_assemble_ex can build (bit flags). */
typedef enum axia_assemble_flags {
  AXIA_ASM_CSR64 = 1,   /* K_ff in CSR, FP64 values (the reference's Csr, linalg.rs:3-8) */
  AXIA_ASM_CSR32 = 2,   /* FP32 copy of the CSR values */
  AXIA_ASM_BSR64 = 4,   /* full-DOF node-block (3x3) form, FP64 */
  AXIA_ASM_BSR32 = 8,   /* full-DOF node-block (3x3) form, FP32 */
  AXIA_ASM_SYM32 = 16,  /* the FP32 node-block form in symmetric storage: each block K_ab, b >= a,
                           stored once (about half the bytes of AXIA_ASM_BSR32) */
  AXIA_ASM_BSR32LO = 32 /* with AXIA_ASM_BSR32: the FP32 low parts K64 - K32 of the node-block
                           values, so K32 + K32lo holds K to 48 bits; axia_gpu_solve_batched then
                           computes its reliable updates B - K X in double-word arithmetic on the
                           FP32 pipe and confirms convergence with an FP64 residual */
} axia_assemble_flags;

typedef enum axia_matrix_format {
  AXIA_FORMAT_CSR = 0,  /* solve on K_ff in CSR */
  AXIA_FORMAT_BSR3 = 1,     /* solve on the node-block form (prescribed DOFs as unit rows) */
  AXIA_FORMAT_BSR3_SYM = 2  /* the same, mixed precision, with the FP32 inner matrix in symmetric
                               storage (AXIA_ASM_SYM32 + AXIA_ASM_BSR64); single system only */
} axia_matrix_format;

typedef enum axia_refine_mode {
  AXIA_REFINE_RESTART = 0,   /* classic iterative refinement: each inner solve restarts from 0 */
  AXIA_REFINE_RELIABLE = 1   /* one FP32 Krylov sequence, FP64 residual replaced at each update */
} axia_refine_mode;

/* A C3D8 / C3D20 mesh.  Node d of node a has full DOF index 3*a + d
 * (solver/src/analysis.rs:152-154 with ndn = 3, model.rs:1220-1232). */
typedef struct axia_mesh {
  int64_t n_nodes;
  const double* coords;    /* [n_nodes][3] */
  int64_t n_elem;
  int32_t nn;              /* nodes per element: 8 (C3D8), 20 (C3D20), 4 (C3D4), 10 (C3D10),
                              6 (C3D6) or 15 (C3D15) */
  int32_t reduced;         /* nn = 20: 1 = C3D20R, 2x2x2 Gauss points (quadratic.rs:100-120);
                              nn = 8: 1 = C3D8R (extra.rs:400-457), 2 = C3D8I (extra.rs:256-388) */
  const int32_t* conn;     /* [n_elem][nn], 0-based node indices, CalculiX node order */
  const double* e_elem;    /* [n_elem] Young's modulus per element, or NULL */
  double e;                /* Young's modulus when e_elem == NULL */
  double nu;               /* Poisson's ratio */
} axia_mesh;

typedef enum axia_preconditioner {
  AXIA_PRECOND_JACOBI = 0,  /* diagonal scaling, as linalg.rs:199-259 */
  AXIA_PRECOND_COARSE = 1   /* two-level: diagonal + a coarse space of the rigid-body modes of
                               subdomains (boxes of about coarse_nodes nodes).  Mixed precision
                               on the node-block form only; no reference counterpart -- the
                               solution is the same, the iteration count drops */
} axia_preconditioner;

typedef enum axia_krylov {
  AXIA_KRYLOV_PER_CASE = 0,  /* batched solves: one CG recurrence per load case (linalg.rs:199-259 each) */
  AXIA_KRYLOV_BLOCK = 1      /* batched solves: one block Krylov space for the 32 cases of a launch
                                (breakdown-free block PCG); same solutions, fewer iterations */
} axia_krylov;

typedef struct axia_solve_opts {
  double rtol;             /* stop when ||r||_2 <= rtol ||b||_2 (reference: 1e-8, linalg.rs:363) */
  int64_t max_iter;        /* <= 0: max(4 n, 200) as linalg.rs:376 */
  int32_t precision;       /* axia_precision */
  int32_t refine_mode;     /* axia_refine_mode (mixed only) */
  double inner_rtol;       /* mixed: residual reduction per refinement step (e.g. 1e-3) */
  int32_t max_outer;       /* mixed: refinement steps allowed */
  int32_t spmv_lanes;      /* lanes per row in the SpMV: 0 = automatic, else 1..32 (power of two) */
  int32_t matrix_format;   /* axia_matrix_format */
  int32_t spmv_vec;        /* node-block form: blocks per lane load (1, 2, 4; 0 = automatic) */
  int32_t preconditioner;  /* axia_preconditioner (0 = Jacobi) */
  int32_t coarse_nodes;    /* AXIA_PRECOND_COARSE: nodes per subdomain (0 = about 512 subdomains, but
                              at least ~13,500 matrix node blocks each: 500 nodes for C3D8; at most
                              682 subdomains per system, in a multi-mesh solve per mesh) */
  int32_t krylov;          /* axia_krylov: batched load cases only (0 = one recurrence per case) */
  int32_t reserved;        /* zero */
} axia_solve_opts;

typedef struct axia_solve_info {
  int64_t n_free;          /* independent DOFs (DofMap n_ind) */
  int64_t nnz;             /* stored entries of K_ff */
  int64_t iters;           /* PCG iterations (FP32 inner iterations for mixed) */
  int64_t outer_iters;     /* refinement steps (mixed), 1 for FP64 */
  double residual;         /* final ||b - K_ff x||_2 as the solver tracks it */
  double bnorm;            /* ||b||_2 of the reduced right-hand side */
  double true_residual;    /* ||b - K_ff x||_2 recomputed in FP64 after the solve */
  double ms_setup;         /* symbolic phase (pattern, DOF map) */
  double ms_assemble;      /* element integration + gather into K_ff */
  double ms_solve;         /* PCG (+ refinement) */
  double ms_pcg_kernel;    /* device time of the persistent PCG kernel launches (CUDA events) */
  int64_t pcg_launches;    /* persistent PCG kernel launches of this solve */
  int64_t bad_index;       /* element / load index of an element error, else -1 */
  int32_t status;          /* axia_status of the call */
  int32_t reserved;
} axia_solve_info;

typedef struct axia_ctx axia_ctx;

/* Library ABI version (AXIA_GPU_ABI_VERSION). */
AXIA_API int32_t axia_gpu_abi_version(void);

/* Creates a context on CUDA device `device`.  Returns NULL and sets *status
 * on failure (no device, CUDA error). */
AXIA_API axia_ctx* axia_gpu_create(int32_t device, int32_t* status);
AXIA_API void axia_gpu_destroy(axia_ctx* ctx);
/* Message of the last failed call on ctx ("" when none). */
AXIA_API const char* axia_gpu_last_error(const axia_ctx* ctx);

/* Batched element_ke (solver/src/elem.rs:344-375 Hex8 / Hex8R / Hex8I /
 * Tet4 arms, :394-411 Wedge6 / Wedge15 arms, :487-495 Hex20 arm, :496 Tet10
 * arm; hex8_stiffness elem.rs:194-219, hex20_stiffness quadratic.rs:122-146,
 * tet4_stiffness elem.rs:221-248, tet10_stiffness quadratic.rs:607-627,
 * hex8r / hex8i extra.rs:256-457, wedge6_stiffness extra.rs:109-132,
 * wedge15_stiffness extra.rs:799-819): for n_elem elements with nn
 * (4, 6, 8, 10, 15, 20) nodes each,
 * xyz[n_elem][nn][3] -> ke[n_elem][3nn][3nn] row-major (DOF order
 * node-major, x y z) and vol[n_elem]; `reduced` as in axia_mesh.
 * e[n_elem] per element.  On an element error *bad_elem holds its index. */
AXIA_API int32_t axia_gpu_element_ke(axia_ctx* ctx, int32_t nn, int32_t reduced, int64_t n_elem,
                            const double* xyz, const double* e, double nu, double* ke,
                            double* vol, int64_t* bad_elem);

/* Batched element stiffness that allocates no GPU memory and needs no
 * context.  No counterpart in the reference: it exists for callers that must
 * not call cudaMalloc -- hosts whose device memory belongs to another
 * allocator or to a budget they may not exceed, and latency-critical loops
 * where an allocation's implicit device synchronization is not acceptable.
 * The arguments, results and error codes of axia_gpu_element_ke (host
 * buffers in and out), on the current CUDA device, for three element kinds
 * only: C3D8 (nn = 8, reduced = 0), C3D20 (nn = 20, reduced = 0) and C3D20R
 * (nn = 20, reduced = 1).  Every other nn, and nn = 8 with reduced != 0
 * (C3D8R / C3D8I) or nn = 20 with reduced other than 0 / 1, returns
 * AXIA_ERR_INVALID_ARG.  Limit: n_elem <= 2048 for nn = 8 and <= 512 for
 * nn = 20 (AXIA_ERR_TOO_LARGE above).  Its device memory is one fixed 16 MiB
 * array per device, held until the process exits; the first call on a device
 * looks up that array's address and uploads the element tables, so make it
 * before any stream capture; calls after cudaDeviceReset are not supported.
 * Calls share the array: calls that overlap on the GPU race (calls within one
 * process are serialized). */
AXIA_API int32_t axia_gpu_element_ke_noalloc(int32_t nn, int32_t reduced, int64_t n_elem, const double* xyz,
                                             const double* e, double nu, double* ke, double* vol,
                                             int64_t* bad_elem);

/* Consistent nodal forces of face pressures added into f_full[3*n_nodes], in
 * list order, on the host (apply_pressure solver/src/analysis.rs:1365-1396 ->
 * hex8_face_pressure elem.rs:891-950 / hex20_face_pressure quadratic.rs:275-315
 * / wedge6_face_pressure extra.rs:184-195 / wedge15_face_pressure
 * extra.rs:869-880).  face is 1..6 (P1..P6; wedges 1..5); positive pressure
 * compresses, except on the wedges' triangles P1 / P2, whose node lists wind
 * the other way (kept as in the reference).  Tetrahedra take no pressure
 * (apply_pressure has no arm for them). */
AXIA_API int32_t axia_face_loads(int32_t nn, int64_t n_nodes, const double* coords, const int32_t* conn,
                        int64_t n_loads, const int64_t* elem, const int32_t* face,
                        const double* p, double* f_full, int64_t* bad_load);

/* Symbolic phase for a mesh and its single-point constraints: uploads the
 * mesh, builds node incidence and adjacency, the independent-DOF numbering
 * (ascending full-DOF order, constraint.rs:103-110) and the CSR pattern of
 * K_ff.  bc_dof/bc_val are full DOF indices and values; a later entry for the
 * same DOF wins (analysis.rs:556-565).  Nodes no element touches are pinned
 * (analysis.rs:2283-2330).  Limits: nn*3 <= 60, nnz(K_ff) < 2^31. */
AXIA_API int32_t axia_gpu_setup(axia_ctx* ctx, const axia_mesh* mesh, int64_t n_bc, const int64_t* bc_dof,
                       const double* bc_val);

/* Numeric phase: element stiffness on the device and deterministic gather
 * into K_ff (values in the reference's element order), the Jacobi diagonal
 * and K_fp u0 (the prescribed-value part of constraint.rs:161-165).
 * precision AXIA_PREC_MIXED also stores an FP32 copy of K_ff. */
AXIA_API int32_t axia_gpu_assemble(axia_ctx* ctx, int32_t precision);

/* As axia_gpu_assemble with an explicit set of matrix forms (axia_assemble_flags).
 * K_fp u0 and the CSR diagonal are always built. */
AXIA_API int32_t axia_gpu_assemble_ex(axia_ctx* ctx, int32_t flags);

/* Static solve: rhs = f_free - K_fp u0, PCG on K_ff, u_full = u0 + T x
 * (reconstruct).  f_full[3*n_nodes] in, u_full[3*n_nodes] out (host). */
AXIA_API int32_t axia_gpu_solve(axia_ctx* ctx, const double* f_full, double* u_full,
                       const axia_solve_opts* opts, axia_solve_info* info);

/* Same with f_full and u_full in device memory (for callers that keep the
 * load and displacement vectors resident on the GPU). */
AXIA_API int32_t axia_gpu_solve_device(axia_ctx* ctx, const double* f_full_dev, double* u_full_dev,
                              const axia_solve_opts* opts, axia_solve_info* info);

/* Runs the context's work on `stream` (a cudaStream_t; NULL restores the
 * context's own stream), so a caller can order it with its own work and time
 * it with events on that stream. */
AXIA_API int32_t axia_gpu_set_stream(axia_ctx* ctx, void* stream);

/* Number of kernels the context has launched so far. */
AXIA_API int64_t axia_gpu_kernel_launches(const axia_ctx* ctx);

/* Diagnostic of the bounded device waits: runs one wait that cannot complete
 * (a single block arriving at a grid barrier sized for two) with a limit of
 * limit_us microseconds (1 .. 10,000,000) and reports what the host saw:
 * *status = AXIA_ERR_TIMEOUT when the wait gave up and recorded it (the
 * expected outcome), *elapsed_ms = the probe kernel's duration.  Barrier and
 * status word are re-armed afterwards, so the context stays usable.  Returns
 * AXIA_OK unless the call itself failed. */
AXIA_API int32_t axia_gpu_check_wait_limit(axia_ctx* ctx, int64_t limit_us, int32_t* status, double* elapsed_ms);

/* Measured FMA throughput of the context's device (no reference counterpart;
 * the denominator of the FP64-bound element kernel's roofline): every thread
 * of a full grid runs independent chains of fused multiply-adds, timed with
 * CUDA events (best of three after one warm-up launch).  precision
 * AXIA_PREC_FP64: double; anything else: float.  *tflops = 2 x FMAs / time. */
AXIA_API int32_t axia_gpu_fma_rate(axia_ctx* ctx, int32_t precision, double* tflops);

/* y = K_ff x on device vectors of n_free entries: FP64 (double x, y) with
 * precision AXIA_PREC_FP64, FP32 (float x, y, the FP32 copy of K_ff) with
 * AXIA_PREC_MIXED.  lanes: CSR lanes per row (0 = automatic).  The matrix
 * product of Csr::matvec (solver/src/linalg.rs:41-50). */
AXIA_API int32_t axia_gpu_spmv_device(axia_ctx* ctx, int32_t precision, const void* x_dev, void* y_dev,
                                      int32_t lanes);

/* y = K x on the full-DOF node-block form (x, y of 3*n_nodes entries,
 * double for AXIA_PREC_FP64, float for AXIA_PREC_MIXED); lanes per block row
 * and blocks per lane load (vec) as in axia_solve_opts, 0 = automatic. */
AXIA_API int32_t axia_gpu_bsr_spmv_device(axia_ctx* ctx, int32_t precision, const void* x_dev, void* y_dev,
                                          int32_t lanes, int32_t vec);

/* y = K x with the FP32 matrix in symmetric storage (AXIA_ASM_SYM32; float x,
 * y of 3*n_nodes entries): each row adds its stored blocks K_ab (b >= a) and
 * the transposes of the blocks K_ba (b < a) that the earlier rows store.
 * lanes per block row: 4, 8, 16 or 0 (automatic).  No reference counterpart
 * (the reference stores K in full CSR, linalg.rs:3-8); same product. */
AXIA_API int32_t axia_gpu_sym_spmv_device(axia_ctx* ctx, const float* x_dev, float* y_dev, int32_t lanes);

/* Stored blocks of the symmetric form (pad blocks included; -1 without a
 * context) and, in *lower_entries, its lower-list entries. */
AXIA_API int64_t axia_gpu_sym_blocks(const axia_ctx* ctx, int64_t* lower_entries);

/* Device times (CUDA events, milliseconds) of the last numeric assembly's two
 * phases: the element stiffness kernels and the gather into the matrix forms
 * (with Dirichlet elimination).  No reference counterpart. */
AXIA_API int32_t axia_gpu_assemble_times(const axia_ctx* ctx, double* ms_element, double* ms_gather);

/* Arithmetic of the C3D8, C3D20 and C3D20R element stiffness, for
 * axia_gpu_element_ke and every later assembly on this context:
 * AXIA_ELEMENT_DWORD (default) runs the Gauss loop on the FP32 pipe in
 * double-word arithmetic (pairs of FP32 numbers with error-free
 * transformations, 48 significant bits; Ke within about 3e-14 of max|Ke| of
 * the exact element stiffness) and the assembly sums the element
 * contributions in double words too; AXIA_ELEMENT_FP64 runs both in FP64 as
 * the reference does (hex8_stiffness elem.rs:194-219, hex20_stiffness
 * quadratic.rs:122-146, analysis.rs:651-668).  GB300 executes FP64 at about
 * 1/75 of its FP32 rate, which bounds the FP64 form.  The other element kinds
 * (C3D4, C3D10, C3D6, C3D15, C3D8R, C3D8I) always use FP64.
 * axia_gpu_element_ke_noalloc uses the default. */
enum axia_element_arith { AXIA_ELEMENT_DWORD = 0, AXIA_ELEMENT_FP64 = 1 };
AXIA_API int32_t axia_gpu_set_element_arith(axia_ctx* ctx, int32_t arith);

/* Number of 3x3 node blocks of the node-block form (node adjacency entries). */
AXIA_API int64_t axia_gpu_node_blocks(const axia_ctx* ctx);

/* Size of the coarse space the last AXIA_PRECOND_COARSE solve used: subdomains
 * and coarse unknowns (6 per subdomain; 0 and 0 before such a solve). */
AXIA_API int32_t axia_gpu_coarse_size(const axia_ctx* ctx, int64_t* n_sub, int64_t* n_coarse);

/* Bilinear element form s_e = u_e^T K_e(E=1) v_e for every element of the
 * mesh of the last setup (u_full, v_full: 3*n_nodes; s: n_elem).  With
 * u = v it is twice the unit-modulus strain energy of each element.
 * No reference counterpart (the reference has no sensitivity code). */
AXIA_API int32_t axia_gpu_element_energy(axia_ctx* ctx, const double* u_full, const double* v_full, double* s);

/* Forward half of the SIMP compliance pair (no reference counterpart):
 * E_e = e0 rho_e^penal on the device, assemble (CSR or node-block by
 * opts->matrix_format and opts->precision), solve K u = f, return u_full and
 * compliance C = f . u.  Keeps rho and u on the device for the backward call.
 * Prescribed displacements must be zero (compliance of a loaded structure). */
AXIA_API int32_t axia_gpu_compliance_forward(axia_ctx* ctx, const double* rho, double penal, double e0,
                                             const double* f_full, double* u_full, double* compliance,
                                             const axia_solve_opts* opts, axia_solve_info* info);

/* Backward half: grad[e] = dC/drho_e = -penal rho_e^(penal-1) e0 u_e^T K_e(1) u_e
 * for all elements, from the state of the last forward call (the adjoint of
 * the self-adjoint compliance problem is -u, so no second solve is needed). */
AXIA_API int32_t axia_gpu_compliance_backward(axia_ctx* ctx, double* grad);

/* Many load cases on the assembled mesh in one persistent launch per 32 of
 * them (the reference solves each load case with its own solve_kff call,
 * linalg.rs:311): F and U are [nrhs][3*n_nodes] host arrays (U = u0 + T x per
 * case), each case runs its own Jacobi-PCG recurrence (alpha, beta,
 * convergence) on the FP32 node-block matrix with FP64 reliable updates
 * (opts->inner_rtol = the residual drop between updates) and stops at
 * opts->rtol.  Needs axia_gpu_assemble_ex(AXIA_ASM_BSR64 | AXIA_ASM_BSR32).
 * rel_res (nrhs entries, may be NULL) receives ||b - K x|| / ||b|| per case. */
AXIA_API int32_t axia_gpu_solve_batched(axia_ctx* ctx, int32_t nrhs, const double* F, double* U,
                                        const axia_solve_opts* opts, axia_solve_info* info, double* rel_res);
AXIA_API int32_t axia_gpu_solve_batched_device(axia_ctx* ctx, int32_t nrhs, const double* F_dev, double* U_dev,
                                               const axia_solve_opts* opts, axia_solve_info* info, double* rel_res);

/* Several independent meshes in one context (no reference counterpart: the
 * reference solves each model on its own).  The meshes (same nn, reduced and
 * nu) are concatenated, node and element indices offset per mesh, and set up
 * as one; bc_dof[k] / bc_val[k] (n_bc[k] entries) are mesh k's own DOF
 * indices.  Assemble afterwards with AXIA_ASM_BSR64 | AXIA_ASM_BSR32.  The
 * concatenated full-DOF vector has mesh k's DOFs at 3 * (first node of k). */
AXIA_API int32_t axia_gpu_setup_multi(axia_ctx* ctx, int32_t n_meshes, const axia_mesh* meshes,
                                      const int64_t* n_bc, const int64_t* const* bc_dof,
                                      const double* const* bc_val);

/* Solves every mesh of axia_gpu_setup_multi in one cooperative launch,
 * replayed from a captured CUDA graph: each mesh gets its own group of blocks
 * and runs its own mixed-precision CG (FP32 node-block CG, FP64 reliable
 * updates every opts->inner_rtol drop) to opts->rtol.  f_full / u_full are the
 * concatenated vectors (host here, device in the _device form).  rel_res and
 * iters (n_meshes entries, may be NULL) receive each mesh's relative
 * residual and iteration count; info->bad_index names a failing mesh. */
AXIA_API int32_t axia_gpu_solve_multi(axia_ctx* ctx, const double* f_full, double* u_full,
                                      const axia_solve_opts* opts, axia_solve_info* info, double* rel_res,
                                      int64_t* iters);
AXIA_API int32_t axia_gpu_solve_multi_device(axia_ctx* ctx, const double* f_full_dev, double* u_full_dev,
                                             const axia_solve_opts* opts, axia_solve_info* info, double* rel_res,
                                             int64_t* iters);

/* Post-solve recovery for the displacement u_full [ndof] of the set-up mesh
 * (replaces the loops after the solve in solve_linear,
 * solver/src/analysis.rs:1027-1035 and 1061-1174):
 *   rf          [ndof]        K u - f over all DOFs (reactions at prescribed
 *                             DOFs); f_full NULL means f = 0
 *   stress      [n_nodes][6]  nodal averaged stresses, Voigt xx yy zz xy yz zx
 *                             (element nodal stresses hex8_nodal_stress
 *                             elem.rs:744-779 / hex20_nodal_stress
 *                             quadratic.rs:148-225, summed per node and
 *                             divided by the node's element count)
 *   strain      [n_nodes][6]  from the averaged stress with modulus e_strain
 *                             and the mesh's nu (engineering shears; the
 *                             reference takes its first material's E)
 *   vm          [n_nodes]     von Mises of the averaged stress (elem.rs:651-660)
 *   elem_stress [n_elem][6]   mean of each element's nodal stresses
 * Any output may be NULL.  Host arrays; the _device form takes device
 * pointers, runs on the context's stream and returns when the work is queued
 * and its status read. */
AXIA_API int32_t axia_gpu_recover(axia_ctx* ctx, const double* u_full, const double* f_full, double e_strain,
                                  double* stress, double* strain, double* vm, double* rf, double* elem_stress);
AXIA_API int32_t axia_gpu_recover_device(axia_ctx* ctx, const double* u_full_dev, const double* f_full_dev,
                                         double e_strain, double* stress, double* strain, double* vm, double* rf,
                                         double* elem_stress);

/* solve_kff on the GPU for callers that build K_ff themselves (replaces
 * solver/src/linalg.rs:311 with the PCG backend, and csr_from_triplets
 * linalg.rs:10-38 before it): n_trips triplets (ti, tj, tv) in the caller's
 * order; entries with ti or tj >= n or tv == 0 (or NaN) are dropped, equal
 * (i, j) are summed in input order after a stable sort, exactly as the
 * reference.  Then Jacobi PCG from x = 0 to ||r|| <= opts->rtol ||rhs||
 * (rtol <= 0: 1e-8 as solve_kff's PCG, linalg.rs:363; max_iter <= 0:
 * max(4n, 200)); opts->precision MIXED runs the FP32 inner / FP64 update
 * solver on an FP32 copy.  x [n] out; info->iters, residual, bnorm,
 * true_residual, nnz.  A negative index is AXIA_ERR_INVALID_ARG (bad_index =
 * the triplet).  Replaces any mesh set up on the context (call
 * axia_gpu_setup again for the mesh path).  opts->matrix_format must be CSR. */
AXIA_API int32_t axia_gpu_solve_triplets(axia_ctx* ctx, int64_t n, int64_t n_trips, const int64_t* ti,
                                         const int64_t* tj, const double* tv, const double* rhs, double* x,
                                         const axia_solve_opts* opts, axia_solve_info* info);

/* The same for a caller's CSR (the reference's Csr: int64 indptr [n+1],
 * indices [nnz], data [nnz], full symmetric storage).  An index outside
 * [0, n) is AXIA_ERR_INVALID_ARG. */
AXIA_API int32_t axia_gpu_solve_csr(axia_ctx* ctx, int64_t n, const int64_t* indptr, const int64_t* indices,
                                    const double* data, const double* rhs, double* x, const axia_solve_opts* opts,
                                    axia_solve_info* info);

/* Picks the node-block layout of the mixed solver's FP32 inner loop (lanes
 * per block row, blocks per lane load) for the assembled mesh by timing each
 * instantiated layout for 40 CG iterations of the persistent kernel, and
 * uses it for later solves whose opts leave spmv_lanes and spmv_vec at 0.
 * cache_path (may be NULL): a text file of JSON lines; a stored choice for
 * the same device and matrix shape is reused without timing, a new one is
 * appended.  Needs axia_gpu_assemble_ex(AXIA_ASM_BSR64 | AXIA_ASM_BSR32).
 * us_per_iter (may be NULL) receives the winner's time per iteration (0 when
 * it came from the cache).  No reference counterpart (the reference has no
 * GPU kernels to tune). */
AXIA_API int32_t axia_gpu_autotune(axia_ctx* ctx, const char* cache_path, int32_t* lanes, int32_t* vec,
                                   double* us_per_iter);

/* Picks the tile of the batched load-case kernel (axia_gpu_solve_batched):
 * load cases per lane (1, 2 or 4; a group of 32 / cases lanes covers the 32
 * cases and a warp runs that many groups over interleaved blocks of a row)
 * and blocks per group and step (their vector rows are all requested before
 * the first is used).  Each instantiated pair runs 30 CG iterations of the
 * 32-case solve on the assembled mesh, timed with CUDA events; the fastest
 * per iteration is used by later batched solves.  cache_path and
 * us_per_iter as in axia_gpu_autotune (one JSON line per choice).  Needs
 * axia_gpu_assemble_ex(AXIA_ASM_BSR64 | AXIA_ASM_BSR32).  No reference
 * counterpart. */
AXIA_API int32_t axia_gpu_autotune_batched(axia_ctx* ctx, const char* cache_path, int32_t* cases_per_lane,
                                           int32_t* blocks_per_step, double* us_per_iter);

/* ---- DOF map with multi-point constraints (constraint.rs:8-136) ---------- */
typedef struct axia_dofmap axia_dofmap;

/* DofMap::build: prescribed DOFs (later entries win, analysis.rs:556-565)
 * and MPCs u_slave = sum_k alpha_k u_master_k + u0 (the reference's Mpc,
 * constraint.rs:8-14; MPC i has masters mpc_master[mpc_ptr[i] ..
 * mpc_ptr[i+1]) with mpc_alpha), into u = u0 + T x with nested slaves
 * expanded and prescribed masters folded into u0, exactly as the reference
 * (last MPC per slave wins, 32 expansion passes, coalesce).  A cyclic MPC or
 * a master outside [0, ndof) is AXIA_ERR_INVALID_ARG; no free DOF, no slave
 * and nothing prescribed is AXIA_ERR_NO_FREE_DOF (constraint.rs:111-113).
 * Host object, no device memory. */
AXIA_API int32_t axia_dofmap_build(int64_t ndof, int64_t n_presc, const int64_t* presc_dof,
                                   const double* presc_val, int64_t n_mpc, const int64_t* mpc_slave,
                                   const int64_t* mpc_ptr, const int64_t* mpc_master, const double* mpc_alpha,
                                   const double* mpc_u0, axia_dofmap** out);
/* Independent DOF count n_ind (-1 for NULL). */
AXIA_API int64_t axia_dofmap_n_ind(const axia_dofmap* map);
/* Copies T (CSR over the ndof full DOFs: t_ptr [ndof+1], t_col / t_val
 * [nnz]), u0 [ndof] and ind_of [ndof] (-1: prescribed or slave); any
 * pointer may be NULL.  Returns nnz(T). */
AXIA_API int64_t axia_dofmap_export(const axia_dofmap* map, int64_t* t_ptr, int64_t* t_col, double* t_val,
                                    double* u0, int64_t* ind_of);
AXIA_API void axia_dofmap_free(axia_dofmap* map);

/* The MPC path of solve_linear (analysis.rs:1018-1025) on the GPU:
 * DofMap::reduce (constraint.rs:138-172) of the caller's full-DOF triplets
 * (ti, tj, tv in the caller's order) and load f_full [ndof], then
 * csr_from_triplets, the PCG of axia_gpu_solve_triplets (opts as there) and
 * reconstruct u_full = u0 + T x (constraint.rs:207-217).  K_ff and the
 * reduced right-hand side equal the reference's bit for bit.  Replaces any
 * mesh set up on the context. */
AXIA_API int32_t axia_gpu_solve_reduced(axia_ctx* ctx, const axia_dofmap* map, int64_t n_trips, const int64_t* ti,
                                        const int64_t* tj, const double* tv, const double* f_full, double* u_full,
                                        const axia_solve_opts* opts, axia_solve_info* info);

/* Sizes of the assembled system: n_free and nnz. */
AXIA_API int32_t axia_gpu_system_size(const axia_ctx* ctx, int64_t* n_free, int64_t* nnz);

/* Copies K_ff (CSR, int32 indices, FP64 values), the Jacobi diagonal and
 * K_fp u0 to host buffers of n_free+1, nnz, nnz, n_free, n_free entries.
 * Any pointer may be NULL. */
AXIA_API int32_t axia_gpu_export_system(const axia_ctx* ctx, int32_t* rowptr, int32_t* col, double* val,
                               double* diag, double* kfu0);

/* Independent-DOF index of every full DOF (-1 = prescribed), n_full entries. */
AXIA_API int32_t axia_gpu_export_dofmap(const axia_ctx* ctx, int32_t* ind_of);

#ifdef __cplusplus
}
#endif

#endif /* AXIA_GPU_H */
