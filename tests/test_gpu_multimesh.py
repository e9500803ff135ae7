"""Independent meshes solved together (axia_gpu_setup_multi /
axia_gpu_solve_multi: one cooperative launch, one CTA group per mesh, replayed
from a CUDA graph): every mesh against its own direct solve and against a
single-mesh GPU solve.  Relative displacement error <= 1e-8 at rtol 1e-10."""
import numpy as np
import pytest

from axia_gpu import _lib, meshgen
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _cubes():
    return meshgen.cube_family(count=7, lo=3, hi=9, seed=11)


def test_multi_mesh_matches_direct_per_mesh(gpu_ctx):
    cubes = _cubes()
    gpu_ctx.setup_multi(cubes).assemble_ex(_lib.ASM_BSR64 | _lib.ASM_BSR32)
    f = np.concatenate([c.cload for c in cubes])
    u, info, rel, its = gpu_ctx.solve_multi(f, rtol=1e-10)
    assert np.all(rel <= 1e-10 * 1.0001) and np.all(its > 0)
    node0 = gpu_ctx.node0
    for k, c in enumerate(cubes):
        uk = u[3 * node0[k]:3 * node0[k + 1]]
        ref = O.solve_static(c, solver=O.SOLVER_CHOLESKY)
        err = np.linalg.norm(uk - ref.u) / np.linalg.norm(ref.u)
        assert err < 1e-8, (k, err)
    # replaying the captured graph gives the same bits; a new load re-uses it
    u2, _, _, its2 = gpu_ctx.solve_multi(f, rtol=1e-10)
    assert np.array_equal(u, u2) and np.array_equal(its, its2)
    u3, _, _, _ = gpu_ctx.solve_multi(2.0 * f, rtol=1e-10)
    assert np.linalg.norm(u3 - 2.0 * u) <= 1e-8 * np.linalg.norm(u3)


def test_multi_mesh_iterations_follow_single_solves(gpu_ctx):
    cubes = _cubes()[:3]
    gpu_ctx.setup_multi(cubes).assemble_ex(_lib.ASM_BSR64 | _lib.ASM_BSR32)
    f = np.concatenate([c.cload for c in cubes])
    u, info, rel, its = gpu_ctx.solve_multi(f, rtol=1e-10)
    for k, c in enumerate(cubes):
        gpu_ctx.setup(c).assemble_ex(_lib.ASM_BSR64 | _lib.ASM_BSR32)
        u1, i1 = gpu_ctx.solve(c.cload, rtol=1e-10, precision=_lib.PREC_MIXED, refine_mode=_lib.REFINE_RELIABLE,
                               inner_rtol=0.01, matrix_format=_lib.FORMAT_BSR3)
        assert abs(int(its[k]) - i1.iters) <= max(3, 0.02 * i1.iters), (k, its[k], i1.iters)


def test_multi_mesh_rejects_mixed_element_types(gpu_ctx):
    with pytest.raises(_lib.AxiaError) as e:
        gpu_ctx.setup_multi([meshgen.patch_c3d8(), meshgen.patch_c3d20()])
    assert e.value.code == _lib.ERR_INVALID_ARG
