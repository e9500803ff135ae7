"""The *STATIC fast path: what solve_linear (solver/src/analysis.rs:548-1035)
hands to the GPU when every element is C3D8 / C3D20 with isotropic material
and only single-point constraints are present.

  loads      -> f_full (CLOAD + DLOAD face pressures, host)
  setup      -> DofMap (prescribed, last BC wins) + CSR pattern of K_ff
  assemble   -> element_ke on the device + deterministic gather into K_ff
  solve      -> rhs = f_free - K_fp u0, PCG, u = u0 + T x (reconstruct)

The result carries the reference's SparseResult fields (linalg.rs:261-266):
x / u, the solver name, iterations and residual.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import _lib as L
from .backend import SparseBackend, apply_env_solver, sparse_backend
from .context import GpuContext


@dataclass
class StaticResult:
    u: np.ndarray            # full displacement vector (3 per node)
    name: str                # solver name as SparseResult.name
    iters: int
    residual: float
    info: dict


def solve_linear(model, backend: SparseBackend | None = None, rtol: float = 1e-8, max_iter: int = 0,
                 ctx: GpuContext | None = None, inner_rtol: float | None = None,
                 refine_mode: int = L.REFINE_RELIABLE, matrix_format: int | None = None,
                 preconditioner: int | None = None) -> StaticResult:
    """Solve the linear-static model on the GPU backend.

    Gpu: FP64 Jacobi-PCG on K_ff in CSR (the reference's method).
    GpuMixed: FP32 inner CG with FP64 refinement (reliable updates by default)
    on the node-block form unless matrix_format says CSR; on the node-block
    form with reliable updates the preconditioner defaults to the two-level one
    (diagonal + subdomain rigid-body modes), else the diagonal."""
    apply_env_solver()
    b = backend if backend is not None else sparse_backend()
    if b == SparseBackend.Auto:
        b = SparseBackend.Gpu
    if not SparseBackend(b).is_gpu():
        raise ValueError(f"backend {SparseBackend(b).as_str()} is not a GPU backend")
    mixed = b == SparseBackend.GpuMixed
    own = ctx is None
    ctx = ctx or GpuContext(0)
    try:
        if matrix_format is None:
            matrix_format = L.FORMAT_BSR3 if mixed else L.FORMAT_CSR
        if inner_rtol is None:
            inner_rtol = 0.1 if refine_mode == L.REFINE_RELIABLE else 1e-3
        if preconditioner is None:
            preconditioner = (L.PRECOND_COARSE if mixed and matrix_format == L.FORMAT_BSR3
                              and refine_mode == L.REFINE_RELIABLE else L.PRECOND_JACOBI)
        ctx.setup(model)
        if matrix_format == L.FORMAT_BSR3:
            ctx.assemble_ex(L.ASM_BSR64 | (L.ASM_BSR32 if mixed else 0))
        else:
            ctx.assemble(L.PREC_MIXED if mixed else L.PREC_FP64)
        f = ctx.load_vector(model)
        u, info = ctx.solve(f, rtol=rtol, max_iter=max_iter, precision=L.PREC_MIXED if mixed else L.PREC_FP64,
                            inner_rtol=inner_rtol, refine_mode=refine_mode, matrix_format=matrix_format,
                            preconditioner=preconditioner)
        fmt = "node-block" if matrix_format == L.FORMAT_BSR3 else "CSR"
        if preconditioner == L.PRECOND_COARSE:
            fmt += ", two-level"
        name = f"GPU PCG (FP32 inner, FP64 refinement, {fmt})" if mixed else f"GPU PCG (FP64, {fmt})"
        return StaticResult(u, name, int(info.iters), float(info.residual), info.as_dict())
    finally:
        if own:
            ctx.close()
