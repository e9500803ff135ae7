"""Bounded device waits: a wait that cannot complete (one block at a grid
barrier sized for two) gives up after its limit, the host reads
AXIA_ERR_TIMEOUT from the status word, and the context keeps working (a solve
on it afterwards matches the oracle).  Nothing here faults or hangs the GPU:
the wait ends by its own limit."""
import numpy as np
import pytest

from axia_gpu import _lib, meshgen
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("limit_us", [2000, 50000])
def test_wait_runs_out_and_reports_timeout(gpu_ctx, limit_us):
    status, ms = gpu_ctx.check_wait_limit(limit_us)
    assert status == _lib.ERR_TIMEOUT
    assert ms >= 0.9 * limit_us / 1000.0
    assert ms < limit_us / 1000.0 + 500.0


def test_context_usable_after_timeout(gpu_ctx):
    status, _ = gpu_ctx.check_wait_limit(1000)
    assert status == _lib.ERR_TIMEOUT
    m = meshgen.cantilever_c3d8(8, 2, 2)
    gpu_ctx.setup(m).assemble()
    f = O.load_vector(m)
    u, info = gpu_ctx.solve(f, rtol=1e-10)
    ref = O.solve_static(m, solver=O.SOLVER_PCG, tol=1e-12)
    assert np.linalg.norm(u - ref.u) <= 1e-8 * np.linalg.norm(ref.u)


def test_wait_limit_rejects_bad_limits(gpu_ctx):
    for bad in (0, -5, 10000001):
        with pytest.raises(_lib.AxiaError):
            gpu_ctx.check_wait_limit(bad)
