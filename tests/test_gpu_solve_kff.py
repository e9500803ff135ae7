"""solve_kff on caller triplets / CSR (axia_gpu_solve_triplets,
axia_gpu_solve_csr): the device csr_from_triplets must give the oracle's
K_ff bit for bit (same additions in the same order), and the PCG must match
the oracle's restated pcg (linalg.rs:199-259) and a direct solve."""
import numpy as np
import pytest

from axia_gpu import _lib, meshgen
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _element_triplets(m):
    """K_ff triplets in the reference's order: elements ascending, Ke row-major,
    zero entries skipped (analysis.rs:651-668), mapped to free indices and
    prescribed rows/columns dropped (DofMap::reduce, constraint.rs:138-172)."""
    free = m.free_mask()
    ind = np.full(m.ndof, -1, np.int64)
    ind[free] = np.arange(free.sum())
    ti, tj, tv = [], [], []
    for e in range(m.n_elem):
        ke, _ = O.element_ke(m.coords[m.conn[e]], float(m.e_elem[e]), m.nu, reduced=m.reduced)
        g = ind[(3 * m.conn[e][:, None] + np.arange(3)).ravel()]
        I, J = np.meshgrid(g, g, indexing="ij")
        keep = (I >= 0) & (J >= 0) & (ke != 0.0)
        ti.append(I[keep])
        tj.append(J[keep])
        tv.append(ke[keep])
    return np.concatenate(ti), np.concatenate(tj), np.concatenate(tv), int(free.sum())


def _csr_from_triplets(n, ti, tj, tv):
    """linalg.rs:10-38 in numpy/Python: filter, stable sort, left-to-right run sums."""
    keep = (ti < n) & (tj < n) & (np.abs(tv) > 0.0)
    ti, tj, tv = ti[keep], tj[keep], tv[keep]
    order = np.argsort(ti * n + tj, kind="stable")
    key = (ti * n + tj)[order]
    vals = tv[order]
    heads = np.flatnonzero(np.r_[True, key[1:] != key[:-1]])
    ends = np.r_[heads[1:], key.shape[0]]
    data = np.empty(heads.shape[0])
    for r, (s, e) in enumerate(zip(heads, ends)):
        v = 0.0
        for q in range(s, e):
            v += vals[q]
        data[r] = v
    rows = key[heads] // n
    indptr = np.zeros(n + 1, np.int64)
    np.add.at(indptr, rows + 1, 1)
    return np.cumsum(indptr), key[heads] % n, data


@pytest.fixture(scope="module")
def cantilever_system():
    m = meshgen.cantilever_c3d8()
    ti, tj, tv, n = _element_triplets(m)
    f = O.load_vector(m)
    rhs = f[m.free_mask()]
    return m, ti, tj, tv, n, rhs


def test_triplets_build_the_oracle_csr_bitwise(gpu_ctx, cantilever_system):
    m, ti, tj, tv, n, rhs = cantilever_system
    ref = O.solve_static(m, solver=O.SOLVER_CHOLESKY, keep_csr=True)
    x, info = gpu_ctx.solve_kff(n, (ti, tj, tv), rhs)
    rp, col, val, dg, _ = gpu_ctx.export_system()
    assert np.array_equal(rp, ref.indptr) and np.array_equal(col, ref.indices)
    assert np.array_equal(val, ref.data)  # same additions, same order
    ip, ix, dv = _csr_from_triplets(n, ti, tj, tv)
    assert np.array_equal(val, dv) and np.array_equal(col, ix)
    assert np.array_equal(dg, val[[np.flatnonzero(col[rp[i]:rp[i + 1]] == i)[0] + rp[i] for i in range(n)]])


def test_triplet_pcg_matches_oracle_pcg_and_direct(gpu_ctx, cantilever_system):
    m, ti, tj, tv, n, rhs = cantilever_system
    x_ref, it_ref, res_ref = O.solve_kff(n, ti, tj, tv, rhs, solver=O.SOLVER_PCG, tol=1e-8)
    x, info = gpu_ctx.solve_kff(n, (ti, tj, tv), rhs)
    assert abs(info.iters - it_ref) <= max(2, 0.02 * it_ref)
    assert info.residual <= 1e-8 * np.linalg.norm(rhs) * 1.0000001
    np.testing.assert_allclose(x, x_ref, rtol=0, atol=1e-6 * np.abs(x_ref).max())
    x_dir, _, _ = O.solve_kff(n, ti, tj, tv, rhs, solver=O.SOLVER_CHOLESKY)
    xt, _ = gpu_ctx.solve_kff(n, (ti, tj, tv), rhs, rtol=1e-12)
    assert np.linalg.norm(xt - x_dir) <= 1e-9 * np.linalg.norm(x_dir)
    xm, im = gpu_ctx.solve_kff(n, (ti, tj, tv), rhs, rtol=1e-10, precision=_lib.PREC_MIXED,
                               refine_mode=_lib.REFINE_RELIABLE, inner_rtol=0.1)
    assert np.linalg.norm(xm - x_dir) <= 1e-8 * np.linalg.norm(x_dir)


def test_csr_entry_equals_triplet_entry(gpu_ctx, cantilever_system):
    m, ti, tj, tv, n, rhs = cantilever_system
    ip, ix, dv = _csr_from_triplets(n, ti, tj, tv)
    x1, i1 = gpu_ctx.solve_kff(n, (ti, tj, tv), rhs, rtol=1e-10)
    x2, i2 = gpu_ctx.solve_csr(n, ip, ix, dv, rhs, rtol=1e-10)
    assert i1.iters == i2.iters
    assert np.array_equal(x1, x2)


def test_dropped_entries_duplicates_and_shuffle(gpu_ctx):
    rng = np.random.default_rng(5)
    n = 300
    a = rng.standard_normal((n, n)) * (rng.random((n, n)) < 0.02)
    k = a @ a.T + n * np.eye(n)
    i, j = np.nonzero(k)
    v = k[i, j]
    # split every entry into 1-3 parts, shuffle, add entries that must be dropped
    parts = rng.integers(1, 4, size=v.shape[0])
    ti = np.repeat(i, parts)
    tj = np.repeat(j, parts)
    w = rng.random(ti.shape[0]) + 0.5
    tv = np.repeat(v, parts) * w / np.repeat(np.add.reduceat(w, np.r_[0, np.cumsum(parts)[:-1]]), parts)
    perm = rng.permutation(ti.shape[0])
    ti, tj, tv = ti[perm], tj[perm], tv[perm]
    ti = np.r_[ti, n, 3, 7, 5]
    tj = np.r_[tj, 2, n + 4, 7, 9]
    tv = np.r_[tv, 1.0, 1.0, 0.0, np.nan]
    rhs = rng.standard_normal(n)
    x, info = gpu_ctx.solve_kff(n, (ti, tj, tv), rhs, rtol=1e-12)
    rp, col, val, _, _ = gpu_ctx.export_system()
    ip, ix, dv = _csr_from_triplets(n, ti, tj, tv)
    assert np.array_equal(rp, ip) and np.array_equal(col, ix) and np.array_equal(val, dv)
    x_ref, _, _ = O.solve_kff(n, ti, tj, tv, rhs, solver=O.SOLVER_CHOLESKY)
    assert np.linalg.norm(x - x_ref) <= 1e-10 * np.linalg.norm(x_ref)


def test_errors_and_context_reuse(gpu_ctx, cantilever_system):
    m, ti, tj, tv, n, rhs = cantilever_system
    bad_i = ti.copy()
    bad_i[17] = -1
    with pytest.raises(_lib.AxiaError) as e:
        gpu_ctx.solve_kff(n, (bad_i, tj, tv), rhs)
    assert e.value.code == _lib.ERR_INVALID_ARG
    bad_rhs = rhs.copy()
    bad_rhs[3] = np.nan
    with pytest.raises(_lib.AxiaError) as e:
        gpu_ctx.solve_kff(n, (ti, tj, tv), bad_rhs)
    assert e.value.code == _lib.ERR_NONFINITE
    # a caller system replaces the mesh: the mesh path refuses until setup runs again
    gpu_ctx.solve_kff(n, (ti, tj, tv), rhs)
    with pytest.raises(_lib.AxiaError) as e:
        gpu_ctx.solve(O.load_vector(m))
    assert e.value.code == _lib.ERR_STATE
    gpu_ctx.setup(m)
    gpu_ctx.assemble(_lib.PREC_FP64)
    u, info = gpu_ctx.solve(O.load_vector(m), rtol=1e-10)
    ref = O.solve_static(m, solver=O.SOLVER_CHOLESKY)
    assert np.linalg.norm(u - ref.u) <= 1e-8 * np.linalg.norm(ref.u)
