"""DofMap::build with multi-point constraints on the library's host side
(axia_dofmap_build) against the oracle's restatement (constraint.rs:26-136):
T, u0 and the independent numbering must be identical, and the error cases
must match (CPU only)."""
import numpy as np
import pytest

from axia_gpu import _lib, meshgen
from axia_gpu.dofmap import DofMap
from oracle import oracle as O


def _compare(ndof, pd, pv, mpcs):
    g = DofMap(ndof, pd, pv, mpcs)
    o = O.DofMap(ndof, pd, pv, mpcs)
    t_ptr, t_col, t_val, u0, ind_of = g.export()
    assert g.n_ind == o.n_ind
    assert np.array_equal(t_ptr, o.t_ptr)
    assert np.array_equal(t_col, o.t_col)
    assert np.array_equal(t_val, o.t_val)
    assert np.array_equal(u0, o.u0)
    return g


def test_prescribed_only_is_the_plain_dof_map():
    m = meshgen.cantilever_c3d8()
    g = _compare(m.ndof, m.bc_dof, m.bc_val, [])
    assert g.n_ind == m.n_free


def test_nested_prescribed_masters_and_last_wins():
    ndof = 30
    pd = np.array([0, 1, 2, 5, 5])
    pv = np.array([0.0, 0.1, -0.2, 0.3, 0.4])        # DOF 5: the last value (0.4) wins
    mpcs = [
        (10, [(11, 0.5), (12, 0.25)], 0.01),          # plain
        (11, [(13, 2.0), (1, 1.0)], 0.0),             # nested into 10, prescribed master 1
        (12, [(14, -1.0)], 0.02),
        (14, [(15, 1.0), (5, -0.5)], 0.0),            # two levels deep, prescribed master 5
        (20, [(21, 1.0)], 0.0),
        (20, [(22, 3.0), (22, -1.0)], 0.5),           # same slave: the last MPC wins, terms coalesce
        (2, [(23, 1.0)], 0.0),                        # slave prescribed: ignored
        (24, [(25, 1e-17)], 0.0),                     # |alpha| <= 1e-16 dropped
        (26, [(27, 1.0), (27, -1.0)], 0.0),           # cancels to an empty row
    ]
    _compare(ndof, pd, pv, mpcs)


def test_cyclic_and_bad_master_are_errors():
    with pytest.raises(_lib.AxiaError) as e:
        DofMap(10, [], [], [(1, [(2, 1.0)], 0.0), (2, [(1, 1.0)], 0.0)])
    assert e.value.code == _lib.ERR_INVALID_ARG
    with pytest.raises(O.OracleError):
        O.DofMap(10, [], [], [(1, [(2, 1.0)], 0.0), (2, [(1, 1.0)], 0.0)])
    with pytest.raises(_lib.AxiaError):
        DofMap(10, [], [], [(1, [(12, 1.0)], 0.0)])


def test_all_dofs_constrained():
    g = _compare(6, np.arange(6), np.linspace(0, 1, 6), [])
    assert g.n_ind == 0


def test_random_mpc_sets_match_the_oracle():
    rng = np.random.default_rng(11)
    for trial in range(20):
        ndof = 60
        pd = rng.choice(ndof, 6, replace=False)
        pv = rng.standard_normal(6)
        mpcs = []
        slaves = rng.choice(ndof, 12, replace=False)
        for k, s in enumerate(slaves):
            # masters only among later slaves or free DOFs: no cycles
            pool = [d for d in range(ndof) if d not in slaves[: k + 1]]
            ms = rng.choice(pool, rng.integers(1, 4), replace=False)
            mpcs.append((int(s), [(int(d), float(rng.standard_normal())) for d in ms], float(rng.standard_normal())))
        _compare(ndof, pd, pv, mpcs)
