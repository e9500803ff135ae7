"""Stress recovery and reactions on the GPU (axia_gpu_recover /
axia_gpu_recover_device; kernels element_recover_kernel and k_recover_nodes).

Both sides take the same displacement field, so differences are round-off
only: nodal stresses, strains, von Mises and element means agree with the
oracle's restatement of hex8_nodal_stress / hex20_nodal_stress and the nodal
averaging of solve_linear to 1e-10 of their largest magnitude; reactions
K u - f to 1e-10 of max|f| (they cancel to ~0 at free DOFs).  The reference's
patch-test pins (mean nodal sxx 210 +- 1e-3 for C3D8, -210 +- 1 for C3D20)
are checked on the GPU's own solve."""
import json
import os

import numpy as np
import pytest

from axia_gpu import _lib, meshgen
from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))


def _check_against_oracle(ctx, m, u, f):
    stress, strain, vm, rf, emean = ctx.recover(u, f)
    s_ref, vm_ref, em_ref = O.nodal_stress(m, u, elem_mean=True)
    e_ref = float(np.asarray(m.e_elem).ravel()[0])
    eps_ref = O.nodal_strain(s_ref, e_ref, m.nu)
    rf_ref = O.reactions(m, u, f)
    smax = np.abs(s_ref).max()
    np.testing.assert_allclose(stress, s_ref, rtol=0, atol=1e-10 * smax)
    np.testing.assert_allclose(vm, vm_ref, rtol=0, atol=1e-10 * smax)
    np.testing.assert_allclose(emean, em_ref, rtol=0, atol=1e-10 * smax)
    np.testing.assert_allclose(strain, eps_ref, rtol=0, atol=1e-10 * np.abs(eps_ref).max())
    fmax = max(np.abs(f).max(), np.abs(rf_ref).max())
    np.testing.assert_allclose(rf, rf_ref, rtol=0, atol=1e-10 * fmax)
    return stress, vm, rf


@pytest.mark.parametrize("name,model", [
    ("c3d8_cantilever", meshgen.cantilever_c3d8()),
    ("c3d8_block_perturbed", meshgen.block_c3d8_pressure(n=6)),
    ("c3d20_block", meshgen.block_c3d20_traction(n=3)),
    ("c3d20r_block", meshgen.block_c3d20_traction(n=3, reduced=True)),
])
def test_recover_matches_oracle(gpu_ctx, name, model):
    ref = O.solve_static(model, solver=O.SOLVER_CHOLESKY)
    gpu_ctx.setup(model)
    _check_against_oracle(gpu_ctx, model, ref.u, ref.f)


def test_recover_golden_cantilever(gpu_ctx):
    m = meshgen.cantilever_c3d8()
    g = GOLD["vectors"]["cantilever_20x4x4"]
    u = np.array(g["u"])
    f = O.load_vector(m)
    gpu_ctx.setup(m)
    stress, _, vm, rf, _ = gpu_ctx.recover(u, f)
    vmax = np.abs(g["vm"]).max()
    np.testing.assert_allclose(vm, g["vm"], rtol=0, atol=1e-10 * vmax)
    np.testing.assert_allclose(stress[:, 0], g["sxx"], rtol=0, atol=1e-10 * vmax)
    np.testing.assert_allclose(rf, g["rf"], rtol=0, atol=1e-10 * np.abs(f).max())


@pytest.mark.parametrize("precision", [_lib.PREC_FP64, _lib.PREC_MIXED])
def test_patch_pins_through_gpu_solve(gpu_ctx, precision):
    pins = GOLD["pins"]
    for model, key in ((meshgen.patch_c3d8(), "patch_c3d8_mean_sxx"), (meshgen.patch_c3d20(), "patch_c3d20_mean_sxx")):
        gpu_ctx.setup(model)
        gpu_ctx.assemble(precision)
        f = gpu_ctx.load_vector(model)
        u, info = gpu_ctx.solve(f, rtol=1e-10, precision=precision)
        stress, _, vm, rf, _ = gpu_ctx.recover(u, f)
        pin = pins[key]
        assert abs(stress[:, 0].mean() - pin["value"]) < pin["tol"], key
        assert vm[0] > 0.0
        # reactions balance the applied load
        for q in range(3):
            assert abs(rf[q::3].sum() + f[q::3].sum()) <= 1e-8 * np.abs(f).sum()


def test_recover_device_pointers_and_errors(gpu_ctx):
    torch = pytest.importorskip("torch")
    m = meshgen.block_c3d8_pressure(n=5)
    ref = O.solve_static(m, solver=O.SOLVER_CHOLESKY)
    gpu_ctx.setup(m)
    stress_h, strain_h, vm_h, rf_h, em_h = gpu_ctx.recover(ref.u, ref.f)
    u = torch.from_numpy(ref.u).cuda()
    f = torch.from_numpy(ref.f).cuda()
    st = torch.empty((m.n_nodes, 6), dtype=torch.float64, device="cuda")
    vm = torch.empty(m.n_nodes, dtype=torch.float64, device="cuda")
    rf = torch.empty(m.ndof, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    gpu_ctx.set_stream(stream.cuda_stream)
    gpu_ctx.recover_device(u.data_ptr(), f.data_ptr(), float(m.e_elem[0]), stress_ptr=st.data_ptr(),
                           vm_ptr=vm.data_ptr(), rf_ptr=rf.data_ptr())
    torch.cuda.synchronize()
    gpu_ctx.set_stream(0)
    # the same kernels on the same inputs: bitwise equal
    assert np.array_equal(st.cpu().numpy(), stress_h)
    assert np.array_equal(vm.cpu().numpy(), vm_h)
    assert np.array_equal(rf.cpu().numpy(), rf_h)
    # f = NULL gives K u
    _, _, _, ku, _ = gpu_ctx.recover(ref.u, None)
    np.testing.assert_allclose(ku - ref.f, rf_h, rtol=0, atol=1e-12 * np.abs(ref.f).max())
    # strain with a non-positive modulus is a material error
    with pytest.raises(RuntimeError, match="MATERIAL|strain"):
        gpu_ctx.recover(ref.u, ref.f, e_strain=0.0)


@pytest.mark.parametrize("key", ["le10_c3d20_syy_D", "le10_c3d20_fine_syy_D"])
@pytest.mark.parametrize("precision", [_lib.PREC_FP64, _lib.PREC_MIXED])
def test_nafems_le10_through_gpu(gpu_ctx, key, precision):
    """The reference's LE10 decks end to end on the GPU: face pressure, C3D20
    assembly, solve, stress recovery; sigma_yy(D) against the oracle and the
    reference's pins (nafems.rs:49-88)."""
    pin = GOLD["pins"][key]
    m = meshgen.from_fixture(os.path.join(os.path.dirname(__file__), "golden", pin["fixture"]))
    ref = O.solve_static(m, solver=O.SOLVER_PCG, tol=1e-12)
    s_ref, _ = O.nodal_stress(m, ref.u)
    gpu_ctx.setup(m)
    f = gpu_ctx.load_vector(m)
    if precision == _lib.PREC_FP64:
        gpu_ctx.assemble(precision)
        u, _ = gpu_ctx.solve(f, rtol=1e-12)
    else:
        gpu_ctx.assemble_ex(_lib.ASM_BSR64 | _lib.ASM_BSR32)
        u, _ = gpu_ctx.solve(f, rtol=1e-12, precision=precision, refine_mode=_lib.REFINE_RELIABLE, inner_rtol=0.1,
                             matrix_format=_lib.FORMAT_BSR3)
    stress, _, _, rf, _ = gpu_ctx.recover(u, f)
    syy = stress[m.node_d, 1]
    assert abs(syy - s_ref[m.node_d, 1]) <= 1e-8 * abs(s_ref[m.node_d, 1])
    assert abs(syy - pin["value"]) <= pin["tol"]
    assert abs(syy - pin["target"]) / abs(pin["target"]) < pin["target_rel_tol"]
