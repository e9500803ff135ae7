"""The CPU oracle against the reference's own known answers (CPU only)."""
import json
import os

import numpy as np
import pytest

from axia_gpu import meshgen
from oracle import oracle as O

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))
PINS = GOLD["pins"]
VEC = GOLD["vectors"]


def _mean_ux(u, nodes_1based):
    return float(np.mean([u[3 * (n - 1)] for n in nodes_1based]))


@pytest.mark.parametrize("solver", [O.SOLVER_CHOLESKY, O.SOLVER_PCG])
def test_patch_c3d8(solver):
    pin = PINS["patch_c3d8_mean_ux"]
    r = O.solve_static(meshgen.patch_c3d8(), solver=solver)
    assert abs(_mean_ux(r.u, pin["nodes_1based"]) - pin["value"]) < pin["tol"]


def test_patch_c3d20():
    pin = PINS["patch_c3d20_mean_ux"]
    r = O.solve_static(meshgen.patch_c3d20(), solver=O.SOLVER_CHOLESKY)
    assert abs(_mean_ux(r.u, pin["nodes_1based"]) - pin["value"]) < pin["tol"]


def test_partition_of_unity():
    n, _ = O.hex20_shape(0.0, 0.0, 0.0)
    assert abs(n.sum() - 1.0) < PINS["hex20_partition_of_unity"]["tol"]
    n, _ = O.quad8_shape(0.0, 0.0)
    assert abs(n.sum() - 1.0) < PINS["quad8_partition_of_unity"]["tol"]
    rng = np.random.default_rng(1)
    for xi, eta, zeta in rng.uniform(-1, 1, (10, 3)):
        n8, dn8 = O.hex8_shape(xi, eta, zeta)
        n20, dn20 = O.hex20_shape(xi, eta, zeta)
        assert abs(n8.sum() - 1) < 1e-14 and abs(n20.sum() - 1) < 1e-14
        assert np.abs(dn8.sum(0)).max() < 1e-14 and np.abs(dn20.sum(0)).max() < 1e-13


def test_element_ke_properties():
    for key, nn in (("hex8_distorted", 8), ("hex20_distorted", 20)):
        g = VEC[key]
        xyz = np.array(g["xyz"])
        ke, vol = O.element_ke(xyz, g["e"], g["nu"])
        # matches the committed regression vector
        assert np.allclose(ke.ravel(), g["ke"], rtol=0, atol=1e-9 * np.abs(ke).max())
        assert abs(vol - g["vol"]) < 1e-12
        # symmetric, rigid-body modes in the null space
        assert np.abs(ke - ke.T).max() < 1e-9 * np.abs(ke).max()
        for d in range(3):
            t = np.zeros(3 * nn)
            t[d::3] = 1.0
            assert np.abs(ke @ t).max() < 1e-8 * np.abs(ke).max()
        rot = np.zeros(3 * nn)
        rot[0::3], rot[1::3] = -xyz[:, 1], xyz[:, 0]
        assert np.abs(ke @ rot).max() < 1e-8 * np.abs(ke).max() * np.abs(xyz).max()


def test_element_errors():
    xyz = np.array(VEC["hex8_distorted"]["xyz"])
    inverted = xyz[[4, 5, 6, 7, 0, 1, 2, 3]]
    with pytest.raises(O.OracleError) as e:
        O.element_ke(inverted, 1.0, 0.3)
    assert e.value.code == 3  # negative Jacobian, elem.rs:208-210
    with pytest.raises(O.OracleError) as e:
        O.element_ke(xyz, 1.0, 0.5)
    assert e.value.code == 4  # nu >= 0.5, elem.rs:42-44
    flat = xyz.copy()
    flat[:, 2] = 0.0
    with pytest.raises(O.OracleError) as e:
        O.element_ke(flat, 1.0, 0.3)
    assert e.value.code == 2  # singular Jacobian, elem.rs:14-16


def test_face_pressure_resultant():
    # a uniform pressure on a planar face: resultant = p * area along the inward normal
    xyz = np.array(VEC["hex8_distorted"]["xyz"])
    fe = np.array(VEC["hex8_face_p4"]["fe"])
    assert np.allclose(O.face_pressure(xyz, 4, 1.0), fe, atol=1e-14)
    cube = (meshgen.HEX20_XI.astype(float) + 1) / 2
    for face, axis, sign in ((2, 2, -1), (4, 0, -1), (1, 2, 1), (6, 0, 1)):
        f = O.face_pressure(cube, face, 3.0).reshape(20, 3)
        assert abs(f[:, axis].sum() - sign * 3.0) < 1e-12
        f8 = O.face_pressure(cube[:8], face, 3.0).reshape(8, 3)
        assert abs(f8[:, axis].sum() - sign * 3.0) < 1e-12


def test_cantilever_pcg_vs_cholesky_vs_superlu():
    m = meshgen.cantilever_c3d8()
    g = VEC["cantilever_20x4x4"]
    ch = O.solve_static(m, solver=O.SOLVER_CHOLESKY, keep_csr=True)
    assert ch.n_free == g["n_free"] == 1500
    assert ch.nnz == g["nnz_kff"] == 88218
    assert np.abs(ch.u - np.array(g["u"])).max() < 1e-12 * np.abs(ch.u).max()
    pc = O.solve_static(m, solver=O.SOLVER_PCG, tol=1e-12)
    assert np.linalg.norm(pc.u - ch.u) / np.linalg.norm(ch.u) < 1e-9
    x = O.direct_solve(ch.indptr, ch.indices, ch.data, ch.rhs)
    free = m.free_mask()
    assert np.linalg.norm(x - ch.u[free]) / np.linalg.norm(x) < 1e-12
    assert O.residual_ok(ch.residual, ch.bnorm)


def test_pcg_failure_modes():
    m = meshgen.cantilever_c3d8(nx=6, ny=2, nz=2)
    with pytest.raises(O.OracleError) as e:
        O.solve_static(m, solver=O.SOLVER_PCG, tol=1e-12, max_iter=3)
    assert e.value.code == 5  # linalg.rs:253-257
    # zero load: x = 0 with zero iterations (linalg.rs:208-216)
    m.cload[:] = 0
    r = O.solve_static(m, solver=O.SOLVER_PCG)
    assert r.iters == 0 and np.all(r.u == 0)


def test_prescribed_nonzero_and_last_bc_wins():
    m = meshgen.cantilever_c3d8(nx=4, ny=2, nz=2)
    tip = np.nonzero(np.isclose(m.coords[:, 0], 4.0))[0]
    # a prescribed tip displacement; the first entry is overridden by the second
    m.bc_dof = np.concatenate([m.bc_dof, 3 * tip, 3 * tip])
    m.bc_val = np.concatenate([m.bc_val, np.full(tip.shape[0], 5.0), np.full(tip.shape[0], 0.01)])
    m.cload[:] = 0
    r = O.solve_static(m, solver=O.SOLVER_CHOLESKY, reactions=True)
    assert np.allclose(r.u[3 * tip], 0.01)
    # reactions at the clamp balance the reactions at the driven face
    assert abs(r.rf[0::3].sum()) < 1e-8 * np.abs(r.rf).max()


def test_patch_stress_pins():
    """Mean nodal sxx of the reference's patch tests (lib.rs:440-446, 764-772)."""
    m = meshgen.patch_c3d8()
    r = O.solve_static(m, solver=O.SOLVER_CHOLESKY)
    s, vm = O.nodal_stress(m, r.u)
    pin = PINS["patch_c3d8_mean_sxx"]
    assert abs(s[:, 0].mean() - pin["value"]) < pin["tol"]
    assert vm[0] > 0.0
    m = meshgen.patch_c3d20()
    r = O.solve_static(m, solver=O.SOLVER_CHOLESKY)
    s, _ = O.nodal_stress(m, r.u)
    pin = PINS["patch_c3d20_mean_sxx"]
    assert abs(s[:, 0].mean() - pin["value"]) < pin["tol"]


def test_reactions_balance_and_golden():
    """K u - f vanishes at free DOFs and the reactions balance the applied load."""
    m = meshgen.cantilever_c3d8()
    r = O.solve_static(m, solver=O.SOLVER_CHOLESKY, reactions=True)
    rf = O.reactions(m, r.u, r.f)
    free = np.ones(m.ndof, bool)
    free[m.bc_dof] = False
    scale = np.abs(r.f).max()
    assert np.abs(rf[free]).max() < 1e-8 * scale
    for q in range(3):
        # rigid translations are in the null space of K: sum of reactions = -sum of loads
        assert abs(rf[q::3].sum() + r.f[q::3].sum()) < 1e-8 * scale * m.n_nodes
    np.testing.assert_allclose(rf, r.rf, rtol=0, atol=1e-9 * scale)
    g = VEC["cantilever_20x4x4"]
    np.testing.assert_allclose(rf, g["rf"], rtol=0, atol=1e-9 * scale)
    s, vm = O.nodal_stress(m, np.array(g["u"]))
    np.testing.assert_allclose(vm, g["vm"], rtol=1e-12, atol=1e-12 * np.abs(vm).max())


@pytest.mark.parametrize("key", ["le10_c3d20_syy_D", "le10_c3d20_fine_syy_D"])
def test_nafems_le10_stress_pin(key):
    """NAFEMS LE10 on the reference's own decks: sigma_yy at node D equals the
    reference's result (README, 2 decimals) and the NAFEMS target within the
    reference test's tolerance (nafems.rs:49-88)."""
    pin = PINS[key]
    m = meshgen.from_fixture(os.path.join(os.path.dirname(__file__), "golden", pin["fixture"]))
    r = O.solve_static(m, solver=O.SOLVER_PCG, tol=1e-12)
    s, _ = O.nodal_stress(m, r.u)
    syy = s[m.node_d, 1]
    assert abs(syy - pin["value"]) <= pin["tol"]
    assert abs(syy - pin["target"]) / abs(pin["target"]) < pin["target_rel_tol"]


def _tet_patch(nn):
    """2x2x2 cube block of tetrahedra stretched by u_x = 0.01 on x = 2 (rigid modes removed)."""
    m = meshgen.block_tet(n=2, nn=nn)
    lat = np.round(m.coords * 2).astype(int)
    x0 = np.nonzero(lat[:, 0] == 0)[0]
    x1 = np.nonzero(lat[:, 0] == 4)[0]
    o = x0[np.argmin(np.abs(m.coords[x0]).sum(1))]
    yax = x0[np.argmax(m.coords[x0, 1] - 10 * np.abs(m.coords[x0, 2]))]
    zax = x0[np.argmax(m.coords[x0, 2] - 10 * np.abs(m.coords[x0, 1]))]
    bc = list(3 * x0) + [3 * o + 1, 3 * o + 2, 3 * yax + 2, 3 * zax + 1]
    vals = [0.0] * len(bc) + [0.01] * len(x1)
    bc += list(3 * x1)
    m.bc_dof = np.array(bc, np.int64)
    m.bc_val = np.array(vals)
    m.cload = np.zeros(m.ndof)
    return m


@pytest.mark.parametrize("nn", [4, 10])
def test_tetrahedra_patch_and_rigid_modes(nn):
    """C3D4 / C3D10 (elem.rs:221-248, quadratic.rs:546-702): six rigid-body modes per
    element and a uniform-strain patch reproduced exactly (sxx = E * 0.01 / 2)."""
    m = _tet_patch(nn)
    ke, vol = O.element_ke(m.coords[m.conn[0]], 210000.0, 0.3)
    w = np.linalg.eigvalsh(ke)
    assert (np.abs(w) < 1e-8 * w.max()).sum() == 6 and vol > 0
    r = O.solve_static(m, solver=O.SOLVER_CHOLESKY)
    s, _ = O.nodal_stress(m, r.u)
    np.testing.assert_allclose(s[:, 0], 1050.0, rtol=1e-10)
    np.testing.assert_allclose(s[:, 1:], 0.0, atol=1e-8)


@pytest.mark.parametrize("variant", [1, 2], ids=["C3D8R", "C3D8I"])
def test_hex8_variants_rigid_modes_and_patch(variant):
    """C3D8R / C3D8I (extra.rs:256-472): six rigid-body modes, and the C3D8
    patch test (lib.rs:429-446) reproduced: u_x = 0.01, sxx = 210."""
    m = meshgen.patch_c3d8()
    ke, vol = O.element_ke(m.coords[m.conn[0]], 210000.0, 0.3, reduced=variant)
    w = np.linalg.eigvalsh(ke)
    assert (np.abs(w) < 1e-8 * w.max()).sum() == 6
    m.reduced = variant
    r = O.solve_static(m, solver=O.SOLVER_CHOLESKY)
    pin = PINS["patch_c3d8_mean_ux"]
    assert abs(_mean_ux(r.u, pin["nodes_1based"]) - pin["value"]) < pin["tol"]
    s, _ = O.nodal_stress(m, r.u)
    assert abs(s[:, 0].mean() - 210.0) < 1e-3


def _wedge_patch(nn):
    """2x2x2 block of wedges stretched by u_x = 0.01 on x = 2 (rigid modes removed)."""
    m = meshgen.block_wedge(n=2, nn=nn)
    lat = np.round(m.coords * 2).astype(int)
    x0 = np.nonzero(lat[:, 0] == 0)[0]
    x1 = np.nonzero(lat[:, 0] == 4)[0]
    o = x0[np.argmin(np.abs(m.coords[x0]).sum(1))]
    yax = x0[np.argmax(m.coords[x0, 1] - 10 * np.abs(m.coords[x0, 2]))]
    zax = x0[np.argmax(m.coords[x0, 2] - 10 * np.abs(m.coords[x0, 1]))]
    bc = list(3 * x0) + [3 * o + 1, 3 * o + 2, 3 * yax + 2, 3 * zax + 1]
    vals = [0.0] * len(bc) + [0.01] * len(x1)
    bc += list(3 * x1)
    m.bc_dof = np.array(bc, np.int64)
    m.bc_val = np.array(vals)
    m.dload_elem = np.zeros(0, np.int64)
    m.dload_face = np.zeros(0, np.int32)
    m.dload_p = np.zeros(0)
    return m


@pytest.mark.parametrize("nn", [6, 15], ids=["C3D6", "C3D15"])
def test_wedges_patch_and_rigid_modes(nn):
    """C3D6 / C3D15 (extra.rs:84-182, 701-820): six rigid-body modes per element, the
    volume of a unit half-cube, and a uniform-strain patch reproduced (sxx = E * 0.01 / 2)."""
    m = _wedge_patch(nn)
    ke, vol = O.element_ke(m.coords[m.conn[0]], 210000.0, 0.3)
    w = np.linalg.eigvalsh(ke)
    assert (np.abs(w) < 1e-8 * w.max()).sum() == 6
    assert abs(vol - 0.5) < 1e-14
    r = O.solve_static(m, solver=O.SOLVER_CHOLESKY)
    s, _ = O.nodal_stress(m, r.u)
    np.testing.assert_allclose(s[:, 0], 1050.0, rtol=1e-9)
    np.testing.assert_allclose(s[:, 1:], 0.0, atol=1e-7)


@pytest.mark.parametrize("nn", [6, 15], ids=["C3D6", "C3D15"])
def test_wedge_face_pressure_resultant(nn):
    """Resultant of a uniform pressure p = 2 on each face of the unit wedge with corners
    (1,0), (1,1), (0,0).  The quadrilaterals P3..P5 push inward (-p * outward area);
    the triangle lists of extra.rs:187-188 wind against the positive-Jacobian corner
    order, so on P1 / P2 a positive p pulls outward -- the oracle and the host face
    loads keep that as it is."""
    m = meshgen.block_wedge(n=1, nn=nn)
    xyz = m.coords[m.conn[0]]
    expect = {1: [0, 0, -0.5], 2: [0, 0, 0.5], 3: [-1.0, 0, 0], 4: [1.0, -1.0, 0], 5: [0, 1.0, 0]}
    for face, vec in expect.items():
        fe = O.face_pressure(xyz, face, 2.0).reshape(-1, 3).sum(0)
        np.testing.assert_allclose(fe, 2.0 * np.array(vec), atol=1e-13)
    with pytest.raises(O.OracleError):
        O.face_pressure(xyz, 6, 1.0)


@pytest.mark.parametrize("name,model", [("c3d8", meshgen.block_c3d8_pressure(n=6)),
                                        ("c3d20", meshgen.block_c3d20_traction(n=3)),
                                        ("simp", meshgen.simp_beam(nx=6, ny=3, nz=3))])
def test_residual_multi_matches_reactions_and_solutions(name, model):
    """The element-by-element residual K u - f (several vectors, threads) equals
    the serial reactions over the triplets, and is ~0 on the free DOFs of the
    oracle's own direct solution."""
    f = O.load_vector(model)
    rng = np.random.default_rng(3)
    U = rng.standard_normal((3, model.ndof))
    R = O.residual_multi(model, U, f, nthreads=4)
    for k in range(3):
        ref = O.reactions(model, U[k], f)
        assert np.abs(R[k] - ref).max() <= 1e-12 * np.abs(ref).max(), (name, k)
    assert np.array_equal(O.residual_multi(model, U[1], f, nthreads=1), O.residual_multi(model, U[1], f, 1))
    r = O.solve_static(model, solver=O.SOLVER_CHOLESKY, f=f)
    assert O.relative_residual(model, r.u, f, 3) <= 1e-12
