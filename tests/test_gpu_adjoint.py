"""SIMP compliance gradient on the GPU (axia_gpu_compliance_forward /
axia_gpu_compliance_backward, element kernel element_energy_kernel).

The reference has no adjoint code; the checks are (1) the element bilinear
form u_e^T K_e(1) v_e against the oracle's restated hex8/hex20 stiffness,
(2) dC/drho against the oracle's CPU FP64 analytic gradient, (3) central
finite differences with h = 1e-6: the direct difference (C(rho+h) -
C(rho-h)) / 2h, whose FP64 round-off floor is about eps * C / h, and the same
central difference evaluated without cancellation through the exact identity
C(rho+h) - C(rho-h) = -(E(rho+h) - E(rho-h)) u+_e^T K_e(1) u-_e, which must
agree to 1e-6 relative."""
import numpy as np
import pytest

from axia_gpu import _lib, meshgen
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _ke1(model, k):
    ke, _ = O.element_ke(model.coords[model.conn[k]], 1.0, model.nu, reduced=model.reduced)
    return ke


def _edofs(model, k):
    return (3 * model.conn[k][:, None] + np.arange(3)).ravel()


@pytest.mark.parametrize("model", [meshgen.block_c3d8_pressure(n=5), meshgen.block_c3d20_traction(n=3),
                                   meshgen.block_c3d20_traction(n=2, reduced=True)])
def test_element_energy_matches_oracle(gpu_ctx, model):
    gpu_ctx.setup(model)
    rng = np.random.default_rng(3)
    u = rng.standard_normal(model.ndof)
    v = rng.standard_normal(model.ndof)
    s_uv = gpu_ctx.element_energy(u, v)
    s_uu = gpu_ctx.element_energy(u)
    for k in range(model.n_elem):
        ke = _ke1(model, k)
        d = _edofs(model, k)
        ref_uv = u[d] @ ke @ v[d]
        ref_uu = u[d] @ ke @ u[d]
        scale = np.abs(ke).max() * np.abs(u[d]).max() * np.abs(v[d]).max() * ke.shape[0]
        assert abs(s_uv[k] - ref_uv) <= 1e-12 * scale, k
        assert abs(s_uu[k] - ref_uu) <= 1e-12 * abs(ref_uu), k


def test_gradient_matches_oracle_analytic(gpu_ctx):
    m = meshgen.simp_beam(nx=12, ny=6, nz=6)
    gpu_ctx.setup(m)
    f = gpu_ctx.load_vector(m)
    u, c, info = gpu_ctx.compliance_forward(m.rho, m.pexp, m.e0, f, rtol=1e-12)
    g = gpu_ctx.compliance_backward()
    m.e_elem = m.e0 * m.rho ** m.pexp
    ref = O.solve_static(m, solver=O.SOLVER_CHOLESKY, f=f)
    assert abs(c - f @ ref.u) <= 1e-10 * abs(c)
    g_ref = O.compliance_grad(m, m.rho, m.pexp, m.e0, ref.u)
    assert np.abs(g - g_ref).max() <= 1e-9 * np.abs(g_ref).max()
    assert np.all(g < 0)  # stiffening any element lowers the compliance


def test_gradient_matches_central_differences(gpu_ctx):
    m = meshgen.simp_beam(nx=12, ny=6, nz=6)
    gpu_ctx.setup(m)
    f = gpu_ctx.load_vector(m)
    rho, p, e0 = m.rho.copy(), m.pexp, m.e0
    u, c, _ = gpu_ctx.compliance_forward(rho, p, e0, f, rtol=1e-13)
    g = gpu_ctx.compliance_backward()
    h = 1e-6
    rng = np.random.default_rng(20)
    for k in rng.choice(m.n_elem, 6, replace=False):
        rp, rm = rho.copy(), rho.copy()
        rp[k] += h
        rm[k] -= h
        up, cp, _ = gpu_ctx.compliance_forward(rp, p, e0, f, rtol=1e-13)
        um, cm, _ = gpu_ctx.compliance_forward(rm, p, e0, f, rtol=1e-13)
        d = _edofs(m, k)
        dc = -(e0 * rp[k] ** p - e0 * rm[k] ** p) * (up[d] @ _ke1(m, k) @ um[d])
        fd_exact = dc / (2 * h)
        assert abs(fd_exact - g[k]) <= 1e-6 * abs(g[k]), (k, fd_exact, g[k])
        fd = (cp - cm) / (2 * h)
        floor = 2e3 * np.finfo(float).eps * abs(c) / h
        assert abs(fd - g[k]) <= 1e-6 * abs(g[k]) + floor, (k, fd, g[k])


def test_backward_needs_forward_and_rejects_bad_density(gpu_ctx):
    m = meshgen.simp_beam(nx=4, ny=2, nz=2)
    gpu_ctx.setup(m)
    with pytest.raises(_lib.AxiaError) as e:
        gpu_ctx.compliance_backward()
    assert e.value.code == _lib.ERR_STATE
    rho = m.rho.copy()
    rho[3] = 0.0
    with pytest.raises(_lib.AxiaError) as e:
        gpu_ctx.compliance_forward(rho, 3.0, 1.0, gpu_ctx.load_vector(m))
    assert e.value.code == _lib.ERR_MATERIAL


@pytest.mark.parametrize("fmt,prec", [(_lib.FORMAT_BSR3, _lib.PREC_FP64), (_lib.FORMAT_BSR3, _lib.PREC_MIXED)])
def test_forward_formats_agree(gpu_ctx, fmt, prec):
    m = meshgen.simp_beam(nx=10, ny=5, nz=5)
    gpu_ctx.setup(m)
    f = gpu_ctx.load_vector(m)
    u0, c0, _ = gpu_ctx.compliance_forward(m.rho, m.pexp, m.e0, f, rtol=1e-11)
    g0 = gpu_ctx.compliance_backward()
    u1, c1, _ = gpu_ctx.compliance_forward(m.rho, m.pexp, m.e0, f, rtol=1e-11, matrix_format=fmt, precision=prec,
                                           refine_mode=_lib.REFINE_RELIABLE, inner_rtol=0.1)
    g1 = gpu_ctx.compliance_backward()
    assert abs(c1 - c0) <= 1e-9 * abs(c0)
    assert np.abs(g1 - g0).max() <= 1e-8 * np.abs(g0).max()
