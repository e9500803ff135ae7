"""C3D6 and C3D15 on the GPU (element_ke_kernel<6,6> / <15,9>, recovery
<6,12> / <15,24>, energy <6,6> / <15,9>) against the oracle's restatement of
wedge6_stiffness (extra.rs:109-132), wedge15_stiffness (extra.rs:799-819),
their nodal stresses (extra.rs:134-153, 821-850) and face loads
(extra.rs:184-253, 869-954)."""
import numpy as np
import pytest

from axia_gpu import _lib, meshgen
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _random_wedges(nn, count, seed):
    rng = np.random.default_rng(seed)
    base = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 0], [1, 0, 1], [0, 1, 1], [0, 0, 1]], float)
    out = []
    for _ in range(count):
        c = base * rng.uniform(0.5, 2.0, 3) + rng.uniform(-0.1, 0.1, (6, 3))
        if nn == 15:
            mids = np.array([(c[a] + c[b]) / 2 for a, b in meshgen.WEDGE15_EDGES]) + rng.uniform(-0.02, 0.02, (9, 3))
            c = np.vstack([c, mids])
        out.append(c)
    return np.array(out)


@pytest.mark.parametrize("nn", [6, 15])
def test_element_ke_matches_oracle(gpu_ctx, nn):
    xyz = _random_wedges(nn, 40, seed=nn)
    e = np.linspace(1000.0, 210000.0, xyz.shape[0])
    ke, vol = gpu_ctx.element_ke(xyz, e, 0.3)
    for k in range(xyz.shape[0]):
        ref, v = O.element_ke(xyz[k], e[k], 0.3)
        assert np.abs(ke[k] - ref).max() <= 1e-12 * np.abs(ref).max()
        assert abs(vol[k] - v) <= 1e-13 * v


@pytest.mark.parametrize("nn", [6, 15])
def test_inverted_wedge_is_reported(gpu_ctx, nn):
    xyz = _random_wedges(nn, 5, seed=3)
    # swap the two triangles (and the bottom / top mid-sides): zeta runs downward
    perm = [3, 4, 5, 0, 1, 2] + ([9, 10, 11, 6, 7, 8, 12, 13, 14] if nn == 15 else [])
    xyz[2] = xyz[2][perm]
    with pytest.raises(O.OracleError):
        O.element_ke(xyz[2], 1000.0, 0.3)
    with pytest.raises(_lib.AxiaError) as e:
        gpu_ctx.element_ke(xyz, np.full(5, 1000.0), 0.3)
    assert e.value.code == _lib.ERR_NEG_JACOBIAN
    assert e.value.bad_index == 2


@pytest.mark.parametrize("nn", [6, 15])
@pytest.mark.parametrize("precision", [_lib.PREC_FP64, _lib.PREC_MIXED])
def test_solve_and_recover_match_oracle(gpu_ctx, nn, precision):
    m = meshgen.block_wedge(n=4 if nn == 6 else 3, nn=nn, perturb=0.2)
    ref = O.solve_static(m, solver=O.SOLVER_CHOLESKY, keep_csr=True)
    gpu_ctx.setup(m)
    f = gpu_ctx.load_vector(m)
    np.testing.assert_allclose(f, ref.f, rtol=0, atol=1e-14 * np.abs(ref.f).max())
    if precision == _lib.PREC_FP64:
        gpu_ctx.assemble_ex(_lib.ASM_CSR64)
        u, _ = gpu_ctx.solve(f, rtol=1e-12)
        rp, col, val, _, _ = gpu_ctx.export_system()
        import scipy.sparse as sp
        n = ref.n_free
        A = sp.csr_matrix((val, col, rp), shape=(n, n))
        R = sp.csr_matrix((ref.data, ref.indices, ref.indptr), shape=(n, n))
        Rs, As = R.copy(), A.copy()
        Rs.data[:] = 1.0
        As.data[:] = 1.0
        assert (Rs - Rs.multiply(As)).nnz == 0
        assert abs(A - R).max() <= 1e-12 * np.abs(ref.data).max()
    else:
        gpu_ctx.assemble_ex(_lib.ASM_BSR64 | _lib.ASM_BSR32)
        u, _ = gpu_ctx.solve(f, rtol=1e-10, precision=precision, refine_mode=_lib.REFINE_RELIABLE, inner_rtol=0.1,
                             matrix_format=_lib.FORMAT_BSR3)
    assert np.linalg.norm(u - ref.u) <= 1e-8 * np.linalg.norm(ref.u)
    stress, _, vm, rf, em = gpu_ctx.recover(ref.u, ref.f)
    s_ref, vm_ref, em_ref = O.nodal_stress(m, ref.u, elem_mean=True)
    smax = np.abs(s_ref).max()
    np.testing.assert_allclose(stress, s_ref, rtol=0, atol=1e-10 * smax)
    np.testing.assert_allclose(vm, vm_ref, rtol=0, atol=1e-10 * smax)
    np.testing.assert_allclose(em, em_ref, rtol=0, atol=1e-10 * smax)
    np.testing.assert_allclose(rf, O.reactions(m, ref.u, ref.f), rtol=0, atol=1e-10 * np.abs(ref.f).max())


@pytest.mark.parametrize("nn", [6, 15])
def test_energy_matches_oracle(gpu_ctx, nn):
    m = meshgen.block_wedge(n=2, nn=nn, perturb=0.2)
    gpu_ctx.setup(m)
    rng = np.random.default_rng(5)
    u = rng.standard_normal(m.ndof)
    s = gpu_ctx.element_energy(u)
    for k in range(m.n_elem):
        ke, _ = O.element_ke(m.coords[m.conn[k]], 1.0, m.nu)
        d = (3 * m.conn[k][:, None] + np.arange(3)).ravel()
        ref = u[d] @ ke @ u[d]
        assert abs(s[k] - ref) <= 1e-12 * abs(ref)
