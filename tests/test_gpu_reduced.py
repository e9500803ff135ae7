"""The MPC path of solve_linear on the GPU (axia_gpu_solve_reduced):
DofMap::reduce on the device must give the oracle's K_ff bit for bit, and the
reconstructed displacements must match the oracle's direct solve."""
import numpy as np
import pytest

from axia_gpu import _lib, meshgen
from axia_gpu.dofmap import DofMap
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _tied_cantilever():
    """The 20x4x4 cantilever with the tip face's z DOFs tied to its centre node,
    the centre's x DOF slaved to a node behind it (a nested chain), and a
    prescribed non-zero displacement at a clamped node (u0 enters the rhs)."""
    m = meshgen.cantilever_c3d8()
    tip = [i for i in range(m.n_nodes) if abs(m.coords[i, 0] - 20.0) < 1e-9]
    c = tip[len(tip) // 2]
    behind = int(np.argmin(np.abs(m.coords - (m.coords[c] - [1.0, 0, 0])).sum(axis=1)))
    mpcs = [(3 * n + 2, [(3 * c + 2, 1.0)], 0.0) for n in tip if n != c]
    mpcs.append((3 * c, [(3 * behind, 1.0), (3 * tip[0] + 2, 0.001)], 1e-4))
    bc_dof = np.r_[m.bc_dof, 3 * 0 + 1]
    bc_val = np.r_[m.bc_val, 0.002]
    return m, bc_dof, bc_val, mpcs


def test_reduced_csr_bitwise_and_solution(gpu_ctx):
    m, bc_dof, bc_val, mpcs = _tied_cantilever()
    ti, tj, tv = O.element_triplets(m)
    f = O.load_vector(m)
    om = O.DofMap(m.ndof, bc_dof, bc_val, mpcs)
    u_ref, _, csr, rhs_ref = om.solve(ti, tj, tv, f, solver=O.SOLVER_CHOLESKY)
    dm = DofMap(m.ndof, bc_dof, bc_val, mpcs)
    u, info = gpu_ctx.solve_reduced(dm, (ti, tj, tv), f, rtol=1e-12)
    rp, col, val, _, _ = gpu_ctx.export_system()
    assert np.array_equal(rp, csr[0]) and np.array_equal(col, csr[1])
    assert np.array_equal(val, csr[2])
    assert np.linalg.norm(u - u_ref) <= 1e-9 * np.linalg.norm(u_ref)
    tip = [i for i in range(m.n_nodes) if abs(m.coords[i, 0] - 20.0) < 1e-9]
    assert np.ptp(u[3 * np.array(tip) + 2]) == 0.0  # tied exactly (u = u0 + T x with one master)
    um, _ = gpu_ctx.solve_reduced(dm, (ti, tj, tv), f, rtol=1e-10, precision=_lib.PREC_MIXED,
                                  refine_mode=_lib.REFINE_RELIABLE, inner_rtol=0.1)
    assert np.linalg.norm(um - u_ref) <= 1e-8 * np.linalg.norm(u_ref)


def test_without_mpcs_equals_the_mesh_path(gpu_ctx):
    m = meshgen.block_c3d8_pressure(n=6)
    ti, tj, tv = O.element_triplets(m)
    f = O.load_vector(m)
    u1, i1 = gpu_ctx.solve_reduced(DofMap(m.ndof, m.bc_dof, m.bc_val), (ti, tj, tv), f, rtol=1e-12)
    gpu_ctx.setup(m)
    gpu_ctx.assemble(_lib.PREC_FP64)
    u2, i2 = gpu_ctx.solve(f, rtol=1e-12)
    assert np.linalg.norm(u1 - u2) <= 1e-10 * np.linalg.norm(u2)


def test_everything_constrained_and_bad_triplet(gpu_ctx):
    m = meshgen.cantilever_c3d8()
    ti, tj, tv = O.element_triplets(m)
    f = O.load_vector(m)
    vals = np.linspace(0.0, 1.0, m.ndof)
    u, _ = gpu_ctx.solve_reduced(DofMap(m.ndof, np.arange(m.ndof), vals), (ti, tj, tv), f)
    assert np.array_equal(u, vals)
    bad = ti.copy()
    bad[5] = -3
    with pytest.raises(_lib.AxiaError) as e:
        gpu_ctx.solve_reduced(DofMap(m.ndof, m.bc_dof, m.bc_val), (bad, tj, tv), f)
    assert e.value.code == _lib.ERR_INVALID_ARG
