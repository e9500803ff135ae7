"""C3D8R (one point + hourglass, extra.rs:400-472) and C3D8I (incompatible
modes condensed, extra.rs:256-395) on the GPU against the oracle's
restatement: element stiffness, assembled solves, recovery and the element
energy of the adjoint."""
import numpy as np
import pytest

from axia_gpu import _lib, meshgen
from oracle import oracle as O

pytestmark = pytest.mark.gpu

KIND = {1: "C3D8R", 2: "C3D8I"}


def _random_hexes(count, seed):
    rng = np.random.default_rng(seed)
    base = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float)
    return np.array([base * rng.uniform(0.5, 2.0, 3) + rng.uniform(-0.12, 0.12, (8, 3)) for _ in range(count)])


@pytest.mark.parametrize("variant", [1, 2], ids=["C3D8R", "C3D8I"])
def test_element_ke_matches_oracle(gpu_ctx, variant):
    xyz = _random_hexes(30, seed=variant)
    e = np.linspace(1000.0, 210000.0, xyz.shape[0])
    ke, vol = gpu_ctx.element_ke(xyz, e, 0.3, reduced=variant)
    for k in range(xyz.shape[0]):
        ref, v = O.element_ke(xyz[k], e[k], 0.3, reduced=variant)
        assert np.abs(ke[k] - ref).max() <= 1e-11 * np.abs(ref).max(), (KIND[variant], k)
        assert abs(vol[k] - v) <= 1e-13 * v


@pytest.mark.parametrize("variant", [1, 2], ids=["C3D8R", "C3D8I"])
@pytest.mark.parametrize("precision", [_lib.PREC_FP64, _lib.PREC_MIXED])
def test_solve_recover_energy(gpu_ctx, variant, precision):
    m = meshgen.block_c3d8_pressure(n=5)
    m.reduced = variant
    ref = O.solve_static(m, solver=O.SOLVER_CHOLESKY)
    gpu_ctx.setup(m)
    f = gpu_ctx.load_vector(m)
    if precision == _lib.PREC_FP64:
        gpu_ctx.assemble_ex(_lib.ASM_CSR64)
        u, _ = gpu_ctx.solve(f, rtol=1e-12)
    else:
        gpu_ctx.assemble_ex(_lib.ASM_BSR64 | _lib.ASM_BSR32)
        u, _ = gpu_ctx.solve(f, rtol=1e-10, precision=precision, refine_mode=_lib.REFINE_RELIABLE, inner_rtol=0.1,
                             matrix_format=_lib.FORMAT_BSR3)
    assert np.linalg.norm(u - ref.u) <= 1e-8 * np.linalg.norm(ref.u)
    stress, _, vm, rf, _ = gpu_ctx.recover(ref.u, ref.f)
    s_ref, vm_ref = O.nodal_stress(m, ref.u)
    smax = np.abs(s_ref).max()
    np.testing.assert_allclose(stress, s_ref, rtol=0, atol=1e-10 * smax)
    np.testing.assert_allclose(rf, O.reactions(m, ref.u, ref.f), rtol=0, atol=1e-9 * np.abs(ref.f).max())
    s = gpu_ctx.element_energy(ref.u)
    for k in range(0, m.n_elem, 7):
        ke, _ = O.element_ke(m.coords[m.conn[k]], 1.0, m.nu, reduced=variant)
        d = (3 * m.conn[k][:, None] + np.arange(3)).ravel()
        r = ref.u[d] @ ke @ ref.u[d]
        assert abs(s[k] - r) <= 1e-10 * abs(r)
