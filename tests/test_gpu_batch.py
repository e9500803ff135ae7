"""Batched load cases (axia_gpu_solve_batched): every case against its own
direct solve (SciPy SuperLU on the oracle's K_ff) and against the
single-case GPU solve.  Relative displacement error <= 1e-8 at rtol 1e-10."""
import numpy as np
import pytest

from axia_gpu import _lib, meshgen
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _direct_all(model, F):
    ref = O.solve_static(model, solver=O.SOLVER_PCG, tol=1e-6, keep_csr=True, f=F[0])
    free = model.free_mask()
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    n = ref.n_free
    K = sp.csr_matrix((ref.data, ref.indices, ref.indptr), shape=(n, n)).tocsc()
    lu = spla.splu(K)
    out = np.zeros_like(F)
    for c in range(F.shape[0]):
        out[c][free] = lu.solve(F[c][free])
    return out


def test_batched_cases_match_direct_and_single(gpu_ctx):
    n = 10
    m = meshgen.block_c3d8_multiload(n=n, nrhs=40)
    F = m.cload_batch.copy()
    F[5] = 0.0                       # a case without load converges at once
    gpu_ctx.setup(m).assemble_ex(_lib.ASM_BSR64 | _lib.ASM_BSR32)
    U, info, rel = gpu_ctx.solve_batched(F, rtol=1e-10)
    assert info.iters > 0 and np.all(rel <= 1e-10 * 1.0001)
    ref = _direct_all(m, F)
    for c in range(F.shape[0]):
        if c == 5:
            assert np.all(U[c] == 0.0)
            continue
        err = np.linalg.norm(U[c] - ref[c]) / np.linalg.norm(ref[c])
        assert err < 1e-8, (c, err)
    u1, i1 = gpu_ctx.solve(F[7], rtol=1e-10, precision=_lib.PREC_MIXED, refine_mode=_lib.REFINE_RELIABLE,
                           inner_rtol=0.01, matrix_format=_lib.FORMAT_BSR3)
    assert np.linalg.norm(U[7] - u1) / np.linalg.norm(u1) < 1e-8


def test_batched_needs_node_block_forms(gpu_ctx):
    m = meshgen.block_c3d8_multiload(n=4, nrhs=2)
    gpu_ctx.setup(m).assemble()
    with pytest.raises(_lib.AxiaError) as e:
        gpu_ctx.solve_batched(m.cload_batch)
    assert e.value.code == _lib.ERR_STATE


def test_batched_prescribed_values(gpu_ctx):
    m = meshgen.cantilever_c3d8(nx=6, ny=3, nz=3)
    tip = np.nonzero(np.isclose(m.coords[:, 0], 6.0))[0]
    m.bc_dof = np.concatenate([m.bc_dof, 3 * tip + 2])
    m.bc_val = np.concatenate([m.bc_val, np.full(tip.shape[0], -0.01)])
    F = np.stack([m.cload * s for s in (0.0, 1.0, -2.0)])
    gpu_ctx.setup(m).assemble_ex(_lib.ASM_BSR64 | _lib.ASM_BSR32)
    U, info, rel = gpu_ctx.solve_batched(F, rtol=1e-11)
    for c in range(3):
        ref = O.solve_static(m, solver=O.SOLVER_CHOLESKY, f=F[c])
        assert np.linalg.norm(U[c] - ref.u) / np.linalg.norm(ref.u) < 1e-8, c
        assert np.allclose(U[c][3 * tip + 2], -0.01)


@pytest.mark.parametrize("pre", [dict(), dict(preconditioner=_lib.PRECOND_COARSE, coarse_nodes=150)],
                         ids=["jacobi", "coarse"])
def test_block_pcg_matches_direct_with_fewer_iterations(gpu_ctx, pre):
    """One block Krylov space for the 32 cases of a launch (AXIA_KRYLOV_BLOCK):
    every case (two launches: 40 cases, one of them without load) equals its
    direct solve to 1e-8 at rtol 1e-10, with fewer iterations than the 32
    separate recurrences, and a repeated solve gives the same bits."""
    m = meshgen.block_c3d8_multiload(n=10, nrhs=40)
    F = m.cload_batch.copy()
    F[5] = 0.0
    gpu_ctx.setup(m).assemble_ex(_lib.ASM_BSR64 | _lib.ASM_BSR32)
    U, info, rel = gpu_ctx.solve_batched(F, rtol=1e-10, krylov=_lib.KRYLOV_BLOCK, **pre)
    assert np.all(rel <= 1e-10 * 1.0001)
    ref = _direct_all(m, F)
    for c in range(F.shape[0]):
        if c == 5:
            assert np.all(U[c] == 0.0)
            continue
        err = np.linalg.norm(U[c] - ref[c]) / np.linalg.norm(ref[c])
        assert err < 1e-8, (c, err)
    U1, i1, _ = gpu_ctx.solve_batched(F[:32], rtol=1e-10, **pre)
    Ub, ib, _ = gpu_ctx.solve_batched(F[:32], rtol=1e-10, krylov=_lib.KRYLOV_BLOCK, **pre)
    assert ib.iters < i1.iters, (ib.iters, i1.iters)
    U2, _, _ = gpu_ctx.solve_batched(F, rtol=1e-10, krylov=_lib.KRYLOV_BLOCK, **pre)
    assert np.array_equal(U, U2)


LO = _lib.ASM_BSR64 | _lib.ASM_BSR32 | _lib.ASM_BSR32LO


@pytest.mark.parametrize("pre", [dict(), dict(preconditioner=_lib.PRECOND_COARSE, coarse_nodes=150)],
                         ids=["jacobi", "coarse"])
def test_batched_double_word_updates_match_direct(gpu_ctx, pre):
    """With the FP32 low parts assembled (AXIA_ASM_BSR32LO) the batched solve
    runs in segments and computes its reliable updates R = B - K X in double
    words (FP32 pairs) between them; a case whose double-word residual meets
    its tolerance is confirmed by an FP64 residual.  Every case equals its
    direct solve to 1e-8 at rtol 1e-10, the per-case residual reported is at
    most rtol, the solution matches the FP64-update solve, and a repeated solve
    gives the same bits."""
    m = meshgen.block_c3d8_multiload(n=10, nrhs=40)
    F = m.cload_batch.copy()
    F[5] = 0.0
    gpu_ctx.setup(m).assemble_ex(LO)
    U, info, rel = gpu_ctx.solve_batched(F, rtol=1e-10, **pre)
    U2, info2, rel2 = gpu_ctx.solve_batched(F, rtol=1e-10, **pre)
    assert np.all(rel <= 1e-10 * 1.0001) and info.outer_iters > 0
    assert np.array_equal(U, U2) and np.array_equal(rel, rel2)
    ref = _direct_all(m, F)
    for c in range(F.shape[0]):
        if c == 5:
            assert np.all(U[c] == 0.0)
            continue
        assert np.linalg.norm(U[c] - ref[c]) <= 1e-8 * np.linalg.norm(ref[c]), c
    gpu_ctx.assemble_ex(_lib.ASM_BSR64 | _lib.ASM_BSR32)
    U64, info64, rel64 = gpu_ctx.solve_batched(F, rtol=1e-10, **pre)
    assert np.linalg.norm(U - U64) <= 1e-8 * np.linalg.norm(U64)


def test_batched_double_word_updates_tight_and_ill_conditioned(gpu_ctx):
    """rtol 1e-12, and a slender cantilever whose double-word residual floor
    (about 2^-47 sum |K| |X|) lies above its tolerance: the solve switches to
    FP64 updates and still meets rtol on the FP64 residual."""
    m = meshgen.block_c3d8_multiload(n=8, nrhs=8)
    gpu_ctx.setup(m).assemble_ex(LO)
    U, info, rel = gpu_ctx.solve_batched(m.cload_batch, rtol=1e-12)
    assert np.all(rel <= 1e-12 * 1.0001)
    ref = _direct_all(m, m.cload_batch)
    for c in range(8):
        assert np.linalg.norm(U[c] - ref[c]) <= 1e-9 * np.linalg.norm(ref[c]), c
    cm = meshgen.cantilever_c3d8()
    F = np.stack([cm.cload * s for s in (1.0, -0.5, 2.0)])
    gpu_ctx.setup(cm).assemble_ex(LO)
    U, info, rel = gpu_ctx.solve_batched(F, rtol=1e-10)
    assert np.all(rel <= 1e-10 * 1.0001)
    for c in range(3):
        r = O.solve_static(cm, solver=O.SOLVER_CHOLESKY, f=F[c])
        assert np.linalg.norm(U[c] - r.u) <= 1e-8 * np.linalg.norm(r.u), c


def test_batched_c3d20_matches_direct(gpu_ctx):
    """C3D20 rows (up to 81 node blocks, longer than the SpMV's staged rows of
    28 blocks) against direct solves, three load cases."""
    m = meshgen.block_c3d20_traction(n=3)
    gpu_ctx.setup(m).assemble_ex(_lib.ASM_BSR64 | _lib.ASM_BSR32)
    f = gpu_ctx.load_vector(m)
    rng = np.random.default_rng(11)
    F = np.stack([f, -0.5 * f, f * rng.uniform(0.5, 2.0, f.shape)])
    U, info, rel = gpu_ctx.solve_batched(F, rtol=1e-10)
    assert np.all(rel <= 1e-10 * 1.0001)
    ref = _direct_all(m, F)
    for c in range(F.shape[0]):
        err = np.linalg.norm(U[c] - ref[c]) / np.linalg.norm(ref[c])
        assert err < 1e-8, (c, err)
