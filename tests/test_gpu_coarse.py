"""Two-level preconditioner of the mixed node-block solve (coarse.cu /
coarse.cuh): Jacobi plus a coarse space of the rigid-body modes of
subdomains.  The reference has no such preconditioner -- its CG is
Jacobi-preconditioned (solver/src/linalg.rs:199-259) -- so the bar is the
reference's solution: the direct solve of K_ff (the restated dense Cholesky,
linalg.rs:78-117, or SciPy SuperLU standing in for faer LL^T) to a relative
error <= 1e-8 at rtol 1e-10, with fewer CG iterations than Jacobi."""
import numpy as np
import pytest

from axia_gpu import _lib, meshgen
from oracle import oracle as O

pytestmark = pytest.mark.gpu

MIXED_BSR = dict(precision=_lib.PREC_MIXED, refine_mode=_lib.REFINE_RELIABLE, matrix_format=_lib.FORMAT_BSR3,
                 inner_rtol=0.1)


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _direct(model):
    ref = O.solve_static(model, solver=O.SOLVER_PCG, tol=1e-6, keep_csr=True)
    free = model.free_mask()
    x = O.direct_solve(ref.indptr, ref.indices, ref.data, ref.rhs)
    u = np.zeros(model.ndof)
    for d, v in zip(model.bc_dof, model.bc_val):
        u[d] = v
    u[free] = x
    return u


def _solve(ctx, model, **kw):
    ctx.setup(model)
    ctx.assemble_ex(_lib.ASM_BSR64 | _lib.ASM_BSR32)
    f = ctx.load_vector(model)
    return ctx.solve(f, rtol=1e-10, **MIXED_BSR, **kw)


@pytest.mark.parametrize("name,model,nodes", [
    ("c3d8_16", meshgen.block_c3d8_pressure(n=16), 300),
    ("c3d8_16_one", meshgen.block_c3d8_pressure(n=16), 100000),
    ("c3d20_5", meshgen.block_c3d20_traction(n=5), 200),
    ("simp_20x10x10", meshgen.simp_beam(nx=20, ny=10, nz=10), 250),
    ("cantilever", meshgen.cantilever_c3d8(), 60),
    ("c3d4_6", meshgen.block_tet(n=6, nn=4, perturb=0.2), 60),
    ("c3d10_4", meshgen.block_tet(n=4, nn=10, perturb=0.2), 100),
    ("c3d6_6", meshgen.block_wedge(n=6, nn=6, perturb=0.2), 60),
    ("c3d15_3", meshgen.block_wedge(n=3, nn=15, perturb=0.2), 80),
])
def test_coarse_matches_direct_with_fewer_iterations(gpu_ctx, name, model, nodes):
    u_ref = _direct(model)
    uj, ij = _solve(gpu_ctx, model)
    uc, ic = _solve(gpu_ctx, model, preconditioner=_lib.PRECOND_COARSE, coarse_nodes=nodes)
    assert _rel(uj, u_ref) < 1e-8, name
    assert _rel(uc, u_ref) < 1e-8, name
    assert ic.true_residual <= 2e-10 * ic.bnorm, name
    if nodes < 1000:  # several subdomains
        assert ic.iters < ij.iters, (name, ic.iters, ij.iters)


def test_coarse_is_deterministic_and_follows_reassembly(gpu_ctx):
    m = meshgen.block_c3d8_pressure(n=12)
    gpu_ctx.setup(m)
    gpu_ctx.assemble_ex(_lib.ASM_BSR64 | _lib.ASM_BSR32)
    f = gpu_ctx.load_vector(m)
    kw = dict(rtol=1e-10, preconditioner=_lib.PRECOND_COARSE, coarse_nodes=200, **MIXED_BSR)
    u1, i1 = gpu_ctx.solve(f, **kw)
    u2, i2 = gpu_ctx.solve(f, **kw)
    assert np.array_equal(u1, u2) and i1.iters == i2.iters
    # a stiffer material: the coarse operator is rebuilt with the new K
    m2 = meshgen.block_c3d8_pressure(n=12)
    m2.e_elem = m2.e_elem * np.linspace(1.0, 3.0, m2.n_elem)
    u3, _ = _solve(gpu_ctx, m2, preconditioner=_lib.PRECOND_COARSE, coarse_nodes=200)
    assert _rel(u3, _direct(m2)) < 1e-8


def test_coarse_tiny_and_clamped_subdomains(gpu_ctx):
    # one element: one subdomain with four clamped nodes
    m = meshgen.patch_c3d8()
    ref = O.solve_static(m, solver=O.SOLVER_CHOLESKY)
    u, info = _solve(gpu_ctx, m, preconditioner=_lib.PRECOND_COARSE, coarse_nodes=1)
    assert _rel(u, ref.u) < 1e-8
    # boxes of ~8 nodes: many subdomains lie entirely on the clamped face or hold
    # a single free node (dependent rotations are dropped)
    m = meshgen.cantilever_c3d8(nx=8, ny=3, nz=3)
    u, info = _solve(gpu_ctx, m, preconditioner=_lib.PRECOND_COARSE, coarse_nodes=8)
    assert _rel(u, _direct(m)) < 1e-8


def test_coarse_rejected_outside_the_mixed_node_block_solve(gpu_ctx):
    m = meshgen.block_c3d8_pressure(n=4)
    gpu_ctx.setup(m)
    gpu_ctx.assemble_ex(_lib.ASM_BSR64 | _lib.ASM_BSR32 | _lib.ASM_CSR64)
    f = gpu_ctx.load_vector(m)
    for kw in (dict(matrix_format=_lib.FORMAT_BSR3), dict(precision=_lib.PREC_MIXED),
               dict(precision=_lib.PREC_FP64, matrix_format=_lib.FORMAT_CSR)):
        with pytest.raises(_lib.AxiaError) as e:
            gpu_ctx.solve(f, preconditioner=_lib.PRECOND_COARSE, **kw)
        assert e.value.code == _lib.ERR_INVALID_ARG
    u, _ = gpu_ctx.solve(f, rtol=1e-10, **MIXED_BSR)  # context still usable
    assert np.all(np.isfinite(u))


def test_batched_load_cases_with_the_coarse_space(gpu_ctx):
    """The 32-column kernel (batch.cu) with the same preconditioner: every case
    against the Jacobi batched solve and its own direct solve, 40 cases (two
    launches, the second with 8 columns), one case without load."""
    m = meshgen.block_c3d8_multiload(n=12, nrhs=40)
    F = m.cload_batch.copy()
    F[5] = 0.0
    gpu_ctx.setup(m).assemble_ex(_lib.ASM_BSR64 | _lib.ASM_BSR32)
    Uj, ij, _ = gpu_ctx.solve_batched(F, rtol=1e-10)
    Uc, ic, rel = gpu_ctx.solve_batched(F, rtol=1e-10, preconditioner=_lib.PRECOND_COARSE, coarse_nodes=150)
    assert np.all(rel <= 1e-10 * 1.0001)
    assert ic.iters < ij.iters, (ic.iters, ij.iters)
    assert np.all(Uc[5] == 0.0)
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    ref = O.solve_static(m, solver=O.SOLVER_PCG, tol=1e-6, keep_csr=True, f=F[0])
    free = m.free_mask()
    lu = spla.splu(sp.csr_matrix((ref.data, ref.indices, ref.indptr), shape=(ref.n_free, ref.n_free)).tocsc())
    for c in range(F.shape[0]):
        if c == 5:
            continue
        u = np.zeros(m.ndof)
        u[free] = lu.solve(F[c][free])
        assert _rel(Uc[c], u) < 1e-8, c
        assert _rel(Uc[c], Uj[c]) < 1e-8, c


def test_multi_mesh_with_per_mesh_coarse_spaces(gpu_ctx):
    """Independent meshes in one launch (multimesh.cu): every mesh gets its own
    subdomains and every CTA group its own chunks and rows of the block-diagonal
    coarse inverse.  Each mesh against its direct solve; fewer iterations than
    the diagonal preconditioner on the larger meshes; graph replay bitwise equal."""
    cubes = meshgen.cube_family(count=6, lo=4, hi=12, seed=5)
    gpu_ctx.setup_multi(cubes).assemble_ex(_lib.ASM_BSR64 | _lib.ASM_BSR32)
    f = np.concatenate([c.cload for c in cubes])
    uj, _, _, itj = gpu_ctx.solve_multi(f, rtol=1e-10)
    u, info, rel, its = gpu_ctx.solve_multi(f, rtol=1e-10, preconditioner=_lib.PRECOND_COARSE, coarse_nodes=60)
    assert np.all(rel <= 1e-10 * 1.0001)
    node0 = gpu_ctx.node0
    for k, c in enumerate(cubes):
        uk = u[3 * node0[k]:3 * node0[k + 1]]
        ref = O.solve_static(c, solver=O.SOLVER_CHOLESKY)
        assert _rel(uk, ref.u) < 1e-8, k
    big = int(np.argmax([c.n_nodes for c in cubes]))
    assert its[big] < itj[big], (its, itj)
    u2, _, _, its2 = gpu_ctx.solve_multi(f, rtol=1e-10, preconditioner=_lib.PRECOND_COARSE, coarse_nodes=60)
    assert np.array_equal(u, u2) and np.array_equal(its, its2)
    # a re-assembly (stiffer material) rebuilds the operator outside the captured graph
    gpu_ctx.assemble_ex(_lib.ASM_BSR64 | _lib.ASM_BSR32)
    u3, _, _, _ = gpu_ctx.solve_multi(2.0 * f, rtol=1e-10, preconditioner=_lib.PRECOND_COARSE, coarse_nodes=60)
    assert np.linalg.norm(u3 - 2.0 * u) <= 1e-8 * np.linalg.norm(u3)


def test_multi_mesh_context_switches_between_block_layouts(gpu_ctx):
    """The multi-mesh solve keeps one block of the coarse inverse per mesh; a
    solve of the same context as one system keeps one block for all meshes.
    Alternating the two rebuilds the space each time; both give the same
    solution (to the solver tolerance) and repeats are bitwise equal."""
    cubes = meshgen.cube_family(count=4, lo=4, hi=9, seed=11)
    gpu_ctx.setup_multi(cubes).assemble_ex(_lib.ASM_BSR64 | _lib.ASM_BSR32)
    f = np.concatenate([c.cload for c in cubes])
    kw = dict(preconditioner=_lib.PRECOND_COARSE, coarse_nodes=40)
    um, _, _, _ = gpu_ctx.solve_multi(f, rtol=1e-11, **kw)
    n_sub_multi, _ = gpu_ctx.coarse_size()
    us, info = gpu_ctx.solve(f, rtol=1e-11, precision=_lib.PREC_MIXED, refine_mode=_lib.REFINE_RELIABLE,
                             matrix_format=_lib.FORMAT_BSR3, **kw)
    assert info.iters > 0
    assert _rel(us, um) < 1e-8
    um2, _, _, _ = gpu_ctx.solve_multi(f, rtol=1e-11, **kw)
    assert np.array_equal(um, um2)
    assert gpu_ctx.coarse_size()[0] == n_sub_multi


def test_many_meshes_share_inversion_groups(gpu_ctx):
    """More meshes than inversion groups (at most 19 of 16 CTAs each on 152
    SMs): groups invert several coarse blocks in turn.  Every mesh against its
    direct solve, repeat bitwise equal."""
    cubes = meshgen.cube_family(count=40, lo=2, hi=6, seed=17)
    gpu_ctx.setup_multi(cubes).assemble_ex(_lib.ASM_BSR64 | _lib.ASM_BSR32)
    f = np.concatenate([c.cload for c in cubes])
    kw = dict(preconditioner=_lib.PRECOND_COARSE, coarse_nodes=40)
    u, info, rel, its = gpu_ctx.solve_multi(f, rtol=1e-11, **kw)
    n_sub, _ = gpu_ctx.coarse_size()
    assert n_sub >= len(cubes)
    node0 = gpu_ctx.node0
    for k, c in enumerate(cubes):
        uk = u[3 * node0[k]:3 * node0[k + 1]]
        ref = O.solve_static(c, solver=O.SOLVER_CHOLESKY)
        # a cube that drew no loaded surface node has u = 0 exactly
        assert np.linalg.norm(uk - ref.u) <= 1e-8 * np.linalg.norm(ref.u), k
    u2, _, _, its2 = gpu_ctx.solve_multi(f, rtol=1e-11, **kw)
    assert np.array_equal(u, u2) and np.array_equal(its, its2)
