"""GPU solutions at sizes well past the direct solve, against the oracle.

The oracle here shares no code with the library: its element stiffness,
assembly (triplets -> DofMap::reduce -> csr_from_triplets) and Jacobi-PCG are
the C++ restatement of solver/src/elem.rs:194-219, quadratic.rs:122-146,
analysis.rs:548-668, constraint.rs:138-172 and linalg.rs:10-38, 199-259,
run here with OpenMP to rtol 1e-13, which stands in for the reference's faer
LL^T (sparse_native.rs:1521-1543) where SciPy SuperLU no longer fits.

Two checks per GPU solution:
* relative displacement error against the oracle's PCG solution:
  <= 1e-9 for the FP64 GPU PCG (solved to rtol 1e-12), <= 1e-8 for the
  mixed forms (solved to rtol 1e-10);
* its residual under the oracle's own stiffness, ||(K_oracle u - f)_free|| /
  ||f_free||, computed element by element without a stored K: <= 1e-9 for
  the rtol 1e-10 solves, <= 1e-11 for the rtol 1e-12 solves.
"""
import os

import numpy as np
import pytest

from axia_gpu import _lib, meshgen
from oracle import oracle as O

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 1
MIXED = dict(precision=_lib.PREC_MIXED, refine_mode=_lib.REFINE_RELIABLE, matrix_format=_lib.FORMAT_BSR3,
             inner_rtol=0.01)
COARSE = dict(MIXED, preconditioner=_lib.PRECOND_COARSE)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _oracle(model, f):
    r = O.solve_static(model, solver=O.SOLVER_PCG, tol=1e-13, nthreads=NT, f=f)
    assert r.residual <= 1e-13 * r.bnorm * 1.0001
    return r.u


def _solve(ctx, model, f, flags, **kw):
    ctx.setup(model)
    ctx.assemble_ex(flags)
    return ctx.solve(f, **kw)


@pytest.mark.parametrize("name,model", [
    ("c3d8_40cubed_perturbed", meshgen.block_c3d8_pressure(n=40)),
    ("c3d20_12cubed", meshgen.block_c3d20_traction(n=12)),
])
def test_fp64_and_mixed_vs_oracle(gpu_ctx, name, model):
    f = O.load_vector(model)
    u_or = _oracle(model, f)
    u64, i64 = _solve(gpu_ctx, model, f, _lib.ASM_CSR64, rtol=1e-12, precision=_lib.PREC_FP64)
    assert _rel(u64, u_or) <= 1e-9, (name, _rel(u64, u_or))
    sols = {"fp64": u64}
    for key, kw in (("mixed", MIXED), ("mixed_coarse", COARSE)):
        u, info = _solve(gpu_ctx, model, f, _lib.ASM_BSR64 | _lib.ASM_BSR32, rtol=1e-10, **kw)
        assert info.true_residual <= 1e-10 * info.bnorm * 1.0001, (name, key)
        assert _rel(u, u_or) <= 1e-8, (name, key, _rel(u, u_or))
        sols[key] = u
    res = O.relative_residual(model, np.stack(list(sols.values())), f, NT)
    assert res[0] <= 1e-11, (name, res)
    assert np.all(res[1:] <= 1e-9), (name, res)


def test_simp_beam_40x20x20_forward_and_gradient_vs_oracle(gpu_ctx):
    m = meshgen.simp_beam(nx=40, ny=20, nz=20)
    f = O.load_vector(m)
    u_or = _oracle(m, f)
    gpu_ctx.setup(m)
    u64, c64, _ = gpu_ctx.compliance_forward(m.rho, m.pexp, m.e0, f, rtol=1e-12)
    assert _rel(u64, u_or) <= 1e-9
    u, c, info = gpu_ctx.compliance_forward(m.rho, m.pexp, m.e0, f, rtol=1e-12, coarse_nodes=0, **COARSE)
    assert _rel(u, u_or) <= 1e-8
    assert abs(c - float(f @ u_or)) <= 1e-8 * abs(c)
    g = gpu_ctx.compliance_backward()
    g_or = O.compliance_grad(m, m.rho, m.pexp, m.e0, u_or)
    assert np.abs(g - g_or).max() <= 1e-8 * np.abs(g_or).max()
    res = O.relative_residual(m, np.stack([u64, u]), f, NT)
    assert np.all(res <= 1e-11), res


def test_batched_32_cases_30cubed_vs_oracle(gpu_ctx):
    m = meshgen.block_c3d8_multiload(n=30, nrhs=32)
    F = m.cload_batch
    gpu_ctx.setup(m).assemble_ex(_lib.ASM_BSR64 | _lib.ASM_BSR32)
    U, info, rel = gpu_ctx.solve_batched(F, rtol=1e-10, preconditioner=_lib.PRECOND_COARSE)
    assert np.all(rel <= 1e-10 * 1.0001)
    res = O.relative_residual(m, U, F, NT)
    assert np.all(res <= 1e-9), res
    for c in (0, 11, 22, 31):
        u_or = _oracle(m, F[c])
        assert _rel(U[c], u_or) <= 1e-8, (c, _rel(U[c], u_or))


def test_multimesh_cubes_up_to_33_vs_oracle(gpu_ctx):
    cubes = meshgen.cube_family(count=3, lo=30, hi=33, seed=5) + meshgen.cube_family(count=3, lo=8, hi=16, seed=6)
    f = np.concatenate([c.cload for c in cubes])
    gpu_ctx.setup_multi(cubes).assemble_ex(_lib.ASM_BSR64 | _lib.ASM_BSR32)
    u, info, rel, its = gpu_ctx.solve_multi(f, rtol=1e-10, preconditioner=_lib.PRECOND_COARSE, coarse_nodes=1000)
    assert np.all(rel <= 1e-10 * 1.0001)
    node0 = gpu_ctx.node0
    assert max(c.shape[0] for c in cubes) >= 30
    for k, c in enumerate(cubes):
        uk = u[3 * node0[k]:3 * node0[k + 1]]
        u_or = _oracle(c, c.cload)
        assert _rel(uk, u_or) <= 1e-8, (k, c.shape, _rel(uk, u_or))
        assert O.relative_residual(c, uk, c.cload, NT) <= 1e-9, k
