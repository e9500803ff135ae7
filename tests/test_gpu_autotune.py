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


BATCH_TILES = {(4, 1), (2, 2), (2, 4), (1, 4), (1, 8)}


def test_batch_autotune_every_tile_solves(gpu_ctx, tmp_path):
    """axia_gpu_autotune_batched picks one of the instantiated tiles of the
    32-case kernel by timing; every tile (forced through a cache entry) gives
    the direct solution of every case to 1e-8 at rtol 1e-10, with and without
    the coarse space."""
    m = meshgen.block_c3d8_multiload(n=12, nrhs=32)
    F = m.cload_batch
    gpu_ctx.setup(m).assemble_ex(_lib.ASM_BSR64 | _lib.ASM_BSR32)
    cache = tmp_path / "batch.jsonl"
    tc, tu, us = gpu_ctx.autotune_batched(str(cache))
    assert (tc, tu) in BATCH_TILES and us > 0
    lines = cache.read_text().splitlines()
    assert len(lines) == 1 and json.loads(lines[0])["cases_per_lane"] == tc
    r = O.solve_static(m, solver=O.SOLVER_PCG, tol=1e-6, keep_csr=True, f=F[0])
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    lu = spla.splu(sp.csr_matrix((r.data, r.indices, r.indptr), shape=(r.n_free, r.n_free)).tocsc())
    free = m.free_mask()
    ref = np.zeros_like(F)
    for c in range(F.shape[0]):
        ref[c][free] = lu.solve(F[c][free])
    entry = json.loads(lines[0])
    for tile in sorted(BATCH_TILES):
        entry["cases_per_lane"], entry["blocks_per_step"] = tile
        cache.write_text(json.dumps(entry) + "\n")
        assert gpu_ctx.autotune_batched(str(cache)) == (tile[0], tile[1], 0.0)
        for pre in (dict(), dict(preconditioner=_lib.PRECOND_COARSE, coarse_nodes=200)):
            U, info, rel = gpu_ctx.solve_batched(F, rtol=1e-10, **pre)
            assert np.all(rel <= 1e-10 * 1.0001), (tile, pre)
            err = np.linalg.norm(U - ref, axis=1) / np.linalg.norm(ref, axis=1)
            assert err.max() < 1e-8, (tile, pre, err.max())


def test_batch_autotune_needs_node_block_forms(gpu_ctx):
    m = meshgen.cantilever_c3d8()
    gpu_ctx.setup(m)
    gpu_ctx.assemble(_lib.PREC_FP64)
    with pytest.raises(_lib.AxiaError) as e:
        gpu_ctx.autotune_batched()
    assert e.value.code == _lib.ERR_STATE
