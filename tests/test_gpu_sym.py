"""The FP32 node-block matrix in symmetric storage (AXIA_ASM_SYM32): each block
K_ab with b >= a stored once, the blocks b < a read transposed from the row
that stores them.  The product is the same K x as the full node-block form
(Csr::matvec, solver/src/linalg.rs:41-50, on the full-DOF system), summed in
another order: FP32 results agree to 1e-6 of the largest |y|, and to the
FP64 product within FP32 rounding.  The mixed solve on it (format
AXIA_FORMAT_BSR3_SYM) reaches the direct solution of K_ff to 1e-8 at rtol
1e-10 like the full form, and repeats bit for bit."""
import numpy as np
import pytest
import torch

from axia_gpu import _lib, meshgen
from oracle import oracle as O

pytestmark = pytest.mark.gpu
ALL = _lib.ASM_BSR64 | _lib.ASM_BSR32 | _lib.ASM_SYM32
MIXED = dict(precision=_lib.PREC_MIXED, refine_mode=_lib.REFINE_RELIABLE, inner_rtol=0.01)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _direct(model):
    ref = O.solve_static(model, solver=O.SOLVER_PCG, tol=1e-6, keep_csr=True)
    u = np.zeros(model.ndof)
    u[model.free_mask()] = O.direct_solve(ref.indptr, ref.indices, ref.data, ref.rhs)
    return u


MODELS = [("c3d8_12", meshgen.block_c3d8_pressure(n=12)),
          ("c3d20_4", meshgen.block_c3d20_traction(n=4)),
          ("c3d4_5", meshgen.block_tet(n=5, nn=4, perturb=0.2)),
          ("cantilever", meshgen.cantilever_c3d8())]


@pytest.mark.parametrize("name,model", MODELS)
def test_sym_structure_and_product(gpu_ctx, name, model):
    gpu_ctx.setup(model).assemble_ex(ALL)
    nadj = gpu_ctx.n_blocks()
    nu, nl = gpu_ctx.sym_blocks()
    assert 2 * nl + model.n_nodes == nadj, name          # every off-diagonal pair once in each list
    assert nadj - nl <= nu <= nadj - nl + model.n_nodes   # upper blocks incl. diagonal, even-padded
    nd = 3 * model.n_nodes
    dev = "cuda:0"
    x64 = torch.randn(nd, dtype=torch.float64, device=dev, generator=torch.Generator(dev).manual_seed(1))
    x32 = x64.float()
    y64 = torch.empty_like(x64)
    ys, yb = torch.empty_like(x32), torch.empty_like(x32)
    gpu_ctx.bsr_spmv_device(_lib.PREC_FP64, x64.data_ptr(), y64.data_ptr())
    gpu_ctx.bsr_spmv_device(_lib.PREC_MIXED, x32.data_ptr(), yb.data_ptr())
    for lanes in (0, 4, 8, 16):
        ys.fill_(float("nan"))
        gpu_ctx.sym_spmv_device(x32.data_ptr(), ys.data_ptr(), lanes)
        torch.cuda.synchronize()
        scale = float(y64.abs().max())
        assert float((ys.double() - yb.double()).abs().max()) <= 1e-6 * scale, (name, lanes)
        assert float((ys.double() - y64).abs().max()) <= 2e-6 * scale, (name, lanes)


@pytest.mark.parametrize("name,model", MODELS[:3])
def test_sym_solve_matches_direct_and_repeats(gpu_ctx, name, model):
    u_ref = _direct(model)
    gpu_ctx.setup(model).assemble_ex(_lib.ASM_BSR64 | _lib.ASM_SYM32)
    f = gpu_ctx.load_vector(model)
    for pre in (dict(), dict(preconditioner=_lib.PRECOND_COARSE, coarse_nodes=100)):
        u1, i1 = gpu_ctx.solve(f, rtol=1e-10, matrix_format=_lib.FORMAT_BSR3_SYM, **MIXED, **pre)
        u2, i2 = gpu_ctx.solve(f, rtol=1e-10, matrix_format=_lib.FORMAT_BSR3_SYM, **MIXED, **pre)
        assert _rel(u1, u_ref) < 1e-8, (name, pre)
        assert i1.true_residual <= 1e-10 * i1.bnorm * 1.0001, (name, pre)
        assert np.array_equal(u1, u2) and i1.iters == i2.iters, (name, pre)


def test_sym_solve_needs_its_forms(gpu_ctx):
    m = meshgen.block_c3d8_pressure(n=4)
    gpu_ctx.setup(m).assemble_ex(_lib.ASM_BSR64 | _lib.ASM_BSR32)
    with pytest.raises(_lib.AxiaError) as e:
        gpu_ctx.solve(gpu_ctx.load_vector(m), rtol=1e-8, matrix_format=_lib.FORMAT_BSR3_SYM, **MIXED)
    assert e.value.code == _lib.ERR_STATE
