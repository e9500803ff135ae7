"""The layout autotuner (axia_gpu_autotune): picks an instantiated
(lanes, blocks per load) pair by timing, the choice changes only the order of
FP32 additions (solutions agree to the solve tolerance), and its JSON-lines
cache is read back instead of timing again."""
import json

import numpy as np
import pytest

from axia_gpu import _lib, meshgen
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CANDIDATES = {(8, 4), (4, 4), (2, 4), (8, 2), (4, 2), (16, 1), (8, 1), (4, 1)}


def test_autotune_choice_cache_and_solution(gpu_ctx, tmp_path):
    m = meshgen.block_c3d8_pressure(n=16)
    gpu_ctx.setup(m)
    gpu_ctx.assemble_ex(_lib.ASM_BSR64 | _lib.ASM_BSR32)
    cache = tmp_path / "layouts.jsonl"
    lanes, vec, us = gpu_ctx.autotune(str(cache))
    assert (lanes, vec) in CANDIDATES and us > 0
    lines = cache.read_text().splitlines()
    assert len(lines) == 1 and json.loads(lines[0])["lanes"] == lanes
    f = gpu_ctx.load_vector(m)
    kw = dict(rtol=1e-10, precision=_lib.PREC_MIXED, refine_mode=_lib.REFINE_RELIABLE, inner_rtol=0.01,
              matrix_format=_lib.FORMAT_BSR3)
    u_tuned, _ = gpu_ctx.solve(f, **kw)
    u_scalar, _ = gpu_ctx.solve(f, spmv_lanes=16, spmv_vec=1, **kw)
    r = O.solve_static(m, solver=O.SOLVER_PCG, tol=1e-6, keep_csr=True)
    ref = np.zeros(m.ndof)
    ref[m.free_mask()] = O.direct_solve(r.indptr, r.indices, r.data, r.rhs)
    for u in (u_tuned, u_scalar):
        assert np.linalg.norm(u - ref) <= 1e-8 * np.linalg.norm(ref)
    # a cached entry is used as stored, without timing
    entry = json.loads(lines[0])
    entry["lanes"], entry["vec"] = 4, 2
    cache.write_text(json.dumps(entry) + "\n")
    lanes2, vec2, us2 = gpu_ctx.autotune(str(cache))
    assert (lanes2, vec2, us2) == (4, 2, 0.0)
    u_cached, _ = gpu_ctx.solve(f, **kw)
    assert np.linalg.norm(u_cached - ref) <= 1e-8 * np.linalg.norm(ref)


def test_autotune_needs_node_block_forms(gpu_ctx):
    m = meshgen.cantilever_c3d8()
    gpu_ctx.setup(m)
    gpu_ctx.assemble(_lib.PREC_FP64)
    with pytest.raises(_lib.AxiaError) as e:
        gpu_ctx.autotune()
    assert e.value.code == _lib.ERR_STATE
