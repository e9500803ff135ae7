"""GPU assembly of K_ff against the oracle's restated path: element loop +
triplet push (solver/src/analysis.rs:574-668), DofMap::reduce
(solver/src/constraint.rs:138-172) and csr_from_triplets (solver/src/linalg.rs:10-38).

Integer parts (DOF map, row pointers, column indices) must match exactly; FP64
values within 1e-12 of max|K| (the element arithmetic is a different but
equivalent closed form, so the last bits differ)."""
import numpy as np
import pytest

from axia_gpu import _lib, meshgen
from oracle import oracle as O

pytestmark = pytest.mark.gpu
VTOL = 1e-12


def _models():
    m_u0 = meshgen.cantilever_c3d8(nx=5, ny=3, nz=2)
    tip = np.nonzero(np.isclose(m_u0.coords[:, 0], 5.0))[0]
    m_u0.bc_dof = np.concatenate([m_u0.bc_dof, 3 * tip + 1])
    m_u0.bc_val = np.concatenate([m_u0.bc_val, np.full(tip.shape[0], 0.02)])
    return [
        ("cantilever_20x4x4", meshgen.cantilever_c3d8()),
        ("block8_6_perturbed", meshgen.block_c3d8_pressure(n=6)),
        ("block20_3", meshgen.block_c3d20_traction(n=3)),
        ("block20r_3", meshgen.block_c3d20_traction(n=3, reduced=True)),
        ("prescribed_nonzero", m_u0),
        ("patch_c3d20", meshgen.patch_c3d20()),
    ]


@pytest.mark.parametrize("name,model", _models(), ids=[n for n, _ in _models()])
def test_kff_matches_oracle(gpu_ctx, name, model):
    ref = O.solve_static(model, solver=O.SOLVER_PCG, tol=1e-6, keep_csr=True)
    gpu_ctx.setup(model).assemble()
    rp, col, val, diag, kfu0 = gpu_ctx.export_system()
    # DOF map: ascending full-DOF order of the free DOFs (constraint.rs:103-110)
    ind = gpu_ctx.export_dofmap()
    free = model.free_mask()
    exp_ind = np.full(model.ndof, -1)
    exp_ind[free] = np.arange(free.sum())
    assert np.array_equal(ind, exp_ind)
    assert gpu_ctx.n_free == ref.n_free
    # the pattern is structural: it equals the oracle's whenever no Ke entry is
    # an exact zero (C3D8), and otherwise holds the oracle's pattern plus entries
    # the reference drops as exact zeros (analysis.rs:658-660, linalg.rs:11)
    import scipy.sparse as sp
    n = ref.n_free
    A = sp.csr_matrix((val, col, rp), shape=(n, n))
    R = sp.csr_matrix((ref.data, ref.indices, ref.indptr), shape=(n, n))
    if model.nn == 8:
        assert np.array_equal(rp.astype(np.int64), ref.indptr), name
        assert np.array_equal(col.astype(np.int64), ref.indices), name
    else:
        Rs = R.copy()
        Rs.data[:] = 1.0
        As = A.copy()
        As.data[:] = 1.0
        assert (Rs - Rs.multiply(As)).nnz == 0, "reference entry missing from the GPU pattern"
    scale = np.abs(ref.data).max()
    assert abs(A - R).max() <= VTOL * scale, name
    # diagonal and the prescribed-value part of the right-hand side
    d_ref = np.array([ref.data[ref.indptr[i]:ref.indptr[i + 1]][ref.indices[ref.indptr[i]:ref.indptr[i + 1]] == i][0]
                      for i in range(ref.n_free)])
    assert np.abs(diag - d_ref).max() <= VTOL * scale
    f = O.load_vector(model)
    rhs_gpu = f[free] - kfu0
    assert np.abs(rhs_gpu - ref.rhs).max() <= 1e-11 * max(1.0, np.abs(ref.rhs).max()), name


def test_assembly_is_bitwise_deterministic(gpu_ctx):
    m = meshgen.block_c3d8_pressure(n=10)
    gpu_ctx.setup(m).assemble()
    a = gpu_ctx.export_system()
    gpu_ctx.assemble()
    b = gpu_ctx.export_system()
    gpu_ctx.setup(m).assemble()
    c = gpu_ctx.export_system()
    for x, y, z in zip(a, b, c):
        assert np.array_equal(x, y) and np.array_equal(x, z)


def test_isolated_node_is_pinned(gpu_ctx):
    # an extra node that no element touches gets all its DOFs pinned (analysis.rs:2283-2330)
    m = meshgen.cantilever_c3d8(nx=3, ny=2, nz=2)
    m.coords = np.vstack([m.coords, [[99.0, 99.0, 99.0]]])
    m.cload = np.concatenate([m.cload, [0.0, 0.0, 0.0]])
    gpu_ctx.setup(m).assemble()
    ind = gpu_ctx.export_dofmap()
    assert np.all(ind[-3:] == -1)
    ref = O.solve_static(m, solver=O.SOLVER_CHOLESKY)
    assert gpu_ctx.n_free == ref.n_free


def test_setup_rejects_bad_input(gpu_ctx):
    m = meshgen.cantilever_c3d8(nx=2, ny=1, nz=1)
    bad = meshgen.cantilever_c3d8(nx=2, ny=1, nz=1)
    bad.conn = bad.conn.copy()
    bad.conn[1, 3] = 10_000
    with pytest.raises(_lib.AxiaError) as e:
        gpu_ctx.setup(bad)
    assert e.value.code == _lib.ERR_INVALID_ARG
    bad = meshgen.cantilever_c3d8(nx=2, ny=1, nz=1)
    bad.bc_dof = np.concatenate([bad.bc_dof, [10 ** 9]])
    bad.bc_val = np.concatenate([bad.bc_val, [0.0]])
    with pytest.raises(_lib.AxiaError) as e:
        gpu_ctx.setup(bad)
    assert e.value.code == _lib.ERR_INVALID_ARG
    bad = meshgen.cantilever_c3d8(nx=2, ny=1, nz=1)
    bad.nu = 0.5
    with pytest.raises(_lib.AxiaError) as e:
        gpu_ctx.setup(bad)
    assert e.value.code == _lib.ERR_MATERIAL
    inv = meshgen.cantilever_c3d8(nx=2, ny=1, nz=1)
    inv.conn = inv.conn[:, [4, 5, 6, 7, 0, 1, 2, 3]].copy()
    gpu_ctx.setup(inv)
    with pytest.raises(_lib.AxiaError) as e:
        gpu_ctx.assemble()
    assert e.value.code == _lib.ERR_NEG_JACOBIAN
    # the context is still usable
    gpu_ctx.setup(m).assemble()


@pytest.mark.parametrize("name,model", _models()[1:4], ids=[n for n, _ in _models()[1:4]])
def test_kff_fp64_element_arith_matches_oracle(gpu_ctx, name, model):
    """The FP64 element arithmetic (AXIA_ELEMENT_FP64) assembles the same K_ff
    within the same tolerance as the default double-word form."""
    ref = O.solve_static(model, solver=O.SOLVER_PCG, tol=1e-6, keep_csr=True)
    gpu_ctx.set_element_arith(_lib.ELEMENT_FP64)
    try:
        gpu_ctx.setup(model).assemble()
        rp, col, val, diag, kfu0 = gpu_ctx.export_system()
    finally:
        gpu_ctx.set_element_arith(_lib.ELEMENT_DWORD)
    import scipy.sparse as sp
    n = ref.n_free
    A = sp.csr_matrix((val, col, rp), shape=(n, n))
    R = sp.csr_matrix((ref.data, ref.indices, ref.indptr), shape=(n, n))
    assert abs(A - R).max() <= VTOL * np.abs(ref.data).max(), name
