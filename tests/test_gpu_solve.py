"""GPU static solve (setup -> assemble -> PCG -> reconstruct) against the
oracle: the restated reference PCG (solver/src/linalg.rs:199-259), the
restated dense Cholesky (linalg.rs:78-117) and SciPy SuperLU standing in for
the reference's faer LL^T.

Tolerances: FP64 PCG at rtol 1e-10 -> relative displacement error vs the
direct solve <= 1e-8 on these conditioning levels, and iteration counts
within 2 % of the oracle's PCG (same algorithm, different rounding).
Mixed precision refined to rtol 1e-10 -> relative error <= 1e-8."""
import json
import os

import numpy as np
import pytest

from axia_gpu import SparseBackend, _lib, meshgen, solve_linear
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _direct(model):
    ref = O.solve_static(model, solver=O.SOLVER_PCG, tol=1e-6, keep_csr=True)
    free = model.free_mask()
    x = O.direct_solve(ref.indptr, ref.indices, ref.data, ref.rhs)
    u = np.zeros(model.ndof)
    for d, v in zip(model.bc_dof, model.bc_val):  # last BC wins
        u[d] = v
    u[free] = x
    return u


@pytest.mark.parametrize("backend", [SparseBackend.Gpu, SparseBackend.GpuMixed])
def test_patch_tests(gpu_ctx, backend):
    pins = GOLD["pins"]
    for model, pin in ((meshgen.patch_c3d8(), pins["patch_c3d8_mean_ux"]),
                       (meshgen.patch_c3d20(), pins["patch_c3d20_mean_ux"])):
        r = solve_linear(model, backend=backend, rtol=1e-12, ctx=gpu_ctx)
        ux = np.mean([r.u[3 * (n - 1)] for n in pin["nodes_1based"]])
        assert abs(ux - pin["value"]) < pin["tol"], (model.name, ux)


def test_cantilever_fp64_matches_oracle(gpu_ctx):
    m = meshgen.cantilever_c3d8()
    g = GOLD["vectors"]["cantilever_20x4x4"]
    u_chol = np.array(g["u"])
    r = solve_linear(m, backend=SparseBackend.Gpu, rtol=1e-10, ctx=gpu_ctx)
    assert _rel(r.u, u_chol) < 1e-8
    ref = O.solve_static(m, solver=O.SOLVER_PCG, tol=1e-10)
    assert abs(r.iters - ref.iters) <= max(2, 0.02 * ref.iters), (r.iters, ref.iters)
    assert _rel(r.u, ref.u) < 1e-9
    assert r.info["true_residual"] <= 1e-9 * r.info["bnorm"]
    # the reference's acceptance rule for a direct solve
    assert O.residual_ok(r.info["true_residual"], r.info["bnorm"])


@pytest.mark.parametrize("name,model", [
    ("block8_12", meshgen.block_c3d8_pressure(n=12)),
    ("block20_5", meshgen.block_c3d20_traction(n=5)),
    ("simp_20x10x10", meshgen.simp_beam(nx=20, ny=10, nz=10)),
])
def test_fp64_and_mixed_vs_direct(gpu_ctx, name, model):
    u_ref = _direct(model)
    r64 = solve_linear(model, backend=SparseBackend.Gpu, rtol=1e-10, ctx=gpu_ctx)
    assert _rel(r64.u, u_ref) < 1e-8, name
    o = O.solve_static(model, solver=O.SOLVER_PCG, tol=1e-10)
    assert abs(r64.iters - o.iters) <= max(3, 0.02 * o.iters), (r64.iters, o.iters)
    for mode, fmt in ((_lib.REFINE_RESTART, _lib.FORMAT_CSR), (_lib.REFINE_RELIABLE, _lib.FORMAT_CSR),
                      (_lib.REFINE_RELIABLE, _lib.FORMAT_BSR3)):
        rmx = solve_linear(model, backend=SparseBackend.GpuMixed, rtol=1e-10, ctx=gpu_ctx, refine_mode=mode,
                           matrix_format=fmt)
        assert _rel(rmx.u, u_ref) < 1e-8, (name, mode, fmt)
        assert rmx.info["outer_iters"] >= 1
        assert rmx.info["true_residual"] <= 2e-10 * rmx.info["bnorm"], (name, mode, fmt)
    # FP64 PCG on the node-block form: same recurrence as on K_ff in CSR
    rb = solve_linear(model, backend=SparseBackend.Gpu, rtol=1e-10, ctx=gpu_ctx, matrix_format=_lib.FORMAT_BSR3)
    assert _rel(rb.u, u_ref) < 1e-8, name
    assert abs(rb.iters - r64.iters) <= max(2, 0.01 * r64.iters), (rb.iters, r64.iters)


def test_solve_is_bitwise_deterministic(gpu_ctx):
    m = meshgen.block_c3d8_pressure(n=10)
    gpu_ctx.setup(m).assemble()
    f = gpu_ctx.load_vector(m)
    u1, i1 = gpu_ctx.solve(f, rtol=1e-10)
    u2, i2 = gpu_ctx.solve(f, rtol=1e-10)
    assert np.array_equal(u1, u2) and i1.iters == i2.iters


def test_zero_load_and_not_converged(gpu_ctx):
    m = meshgen.cantilever_c3d8(nx=6, ny=2, nz=2)
    gpu_ctx.setup(m).assemble()
    u, info = gpu_ctx.solve(np.zeros(m.ndof))
    assert info.iters == 0 and np.all(u == 0)
    with pytest.raises(_lib.AxiaError) as e:
        gpu_ctx.solve(gpu_ctx.load_vector(m), rtol=1e-12, max_iter=3)
    assert e.value.code == _lib.ERR_NOT_CONVERGED
    f = gpu_ctx.load_vector(m)
    f[5] = np.nan
    with pytest.raises(_lib.AxiaError) as e:
        gpu_ctx.solve(f)
    assert e.value.code == _lib.ERR_NONFINITE
    # still usable
    u, info = gpu_ctx.solve(gpu_ctx.load_vector(m), rtol=1e-10)
    assert info.iters > 0


def test_prescribed_displacement_and_reconstruct(gpu_ctx):
    m = meshgen.cantilever_c3d8(nx=5, ny=3, nz=2)
    tip = np.nonzero(np.isclose(m.coords[:, 0], 5.0))[0]
    m.bc_dof = np.concatenate([m.bc_dof, 3 * tip + 2, 3 * tip + 2])
    m.bc_val = np.concatenate([m.bc_val, np.full(tip.shape[0], 9.0), np.full(tip.shape[0], -0.05)])
    m.cload[:] = 0.0
    ref = O.solve_static(m, solver=O.SOLVER_CHOLESKY)
    r = solve_linear(m, backend=SparseBackend.Gpu, rtol=1e-12, ctx=gpu_ctx)
    assert np.allclose(r.u[3 * tip + 2], -0.05)
    assert _rel(r.u, ref.u) < 1e-9


def test_all_dofs_prescribed(gpu_ctx):
    m = meshgen.patch_c3d8()
    m.bc_dof = np.arange(24, dtype=np.int64)
    m.bc_val = np.linspace(0, 1e-3, 24)
    r = solve_linear(m, backend=SparseBackend.Gpu, ctx=gpu_ctx)
    assert np.array_equal(r.u, m.bc_val) and r.iters == 0


@pytest.mark.parametrize("n", [40])
def test_larger_block_properties(gpu_ctx, n):
    """Size-independent properties on a 40^3 perturbed block: true FP64
    residual, symmetry of the solution map (Maxwell-Betti reciprocity) and
    agreement of the FP64 and mixed paths."""
    m = meshgen.block_c3d8_pressure(n=n)
    gpu_ctx.setup(m).assemble(_lib.PREC_MIXED)
    f = gpu_ctx.load_vector(m)
    u64, i64 = gpu_ctx.solve(f, rtol=1e-10)
    assert i64.true_residual <= 1.5e-10 * i64.bnorm
    umx, imx = gpu_ctx.solve(f, rtol=1e-10, precision=_lib.PREC_MIXED)
    assert imx.true_residual <= 1e-10 * imx.bnorm * 1.0001
    assert _rel(umx, u64) < 1e-8
    umr, imr = gpu_ctx.solve(f, rtol=1e-10, precision=_lib.PREC_MIXED, refine_mode=_lib.REFINE_RELIABLE,
                             inner_rtol=0.1)
    assert imr.true_residual <= 1e-10 * imr.bnorm * 1.0001
    assert _rel(umr, u64) < 1e-8
    # one FP32 Krylov sequence needs about as many iterations as FP64 PCG
    assert imr.iters <= 1.3 * i64.iters
    gpu_ctx.assemble_ex(_lib.ASM_CSR64 | _lib.ASM_CSR32 | _lib.ASM_BSR64 | _lib.ASM_BSR32)
    umb, imb = gpu_ctx.solve(f, rtol=1e-10, precision=_lib.PREC_MIXED, refine_mode=_lib.REFINE_RELIABLE,
                             inner_rtol=0.1, matrix_format=_lib.FORMAT_BSR3)
    assert imb.true_residual <= 1e-10 * imb.bnorm * 1.0001
    assert _rel(umb, u64) < 1e-8
    rng = np.random.default_rng(4)
    free = np.nonzero(m.free_mask())[0]
    f1 = np.zeros(m.ndof)
    f2 = np.zeros(m.ndof)
    f1[rng.choice(free, 50)] = rng.standard_normal(50)
    f2[rng.choice(free, 50)] = rng.standard_normal(50)
    u1, _ = gpu_ctx.solve(f1, rtol=1e-12)
    u2, _ = gpu_ctx.solve(f2, rtol=1e-12)
    assert abs(f1 @ u2 - f2 @ u1) <= 1e-9 * abs(f1 @ u2)
