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
                 ctx: GpuContext | None = None, inner_rtol: float = 1e-3,
                 refine_mode: int = L.REFINE_RESTART) -> StaticResult:
    """Solve the linear-static model on the GPU backend (Gpu or GpuMixed)."""
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
        ctx.setup(model)
        ctx.assemble(L.PREC_MIXED if mixed else L.PREC_FP64)
        f = ctx.load_vector(model)
        u, info = ctx.solve(f, rtol=rtol, max_iter=max_iter, precision=L.PREC_MIXED if mixed else L.PREC_FP64,
                            inner_rtol=inner_rtol, refine_mode=refine_mode)
        name = "GPU PCG (FP32 inner, FP64 refinement)" if mixed else "GPU PCG (FP64)"
        return StaticResult(u, name, int(info.iters), float(info.residual), info.as_dict())
    finally:
        if own:
            ctx.close()
