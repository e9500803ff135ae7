"""Host logic on CPU: the C ABI's exported symbols, the host-side load
routine, mesh generators and the solver-selection mirror."""
import ctypes
import os
import re

import numpy as np
import pytest

from axia_gpu import _lib, meshgen
from axia_gpu.backend import (BackendError, SparseBackend, apply_env_solver, parse_sparse_backend,
                              set_sparse_backend, sparse_backend, with_sparse_backend)
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    src = open(os.path.join(ROOT, "include", "axia_gpu.h")).read()
    return sorted(set(re.findall(r"AXIA_API\s+[\w\s\*]+?\b(axia_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    declared = _declared_symbols()
    assert len(declared) >= 13
    for name in declared:
        assert hasattr(lib, name), name
    bound = {n for n, _, _ in _lib.SIGNATURES}
    assert set(declared) == bound, set(declared) ^ bound
    assert lib.axia_gpu_abi_version() == 2


def test_entry_points_reject_null_handles():
    """Every entry point that takes a context (or a DOF map) returns
    AXIA_ERR_INVALID_ARG, -1 for the size getters, for a null handle without
    touching the device; destroy / free accept null."""
    lib = _lib.load()
    defaults = {ctypes.c_int32: 1, ctypes.c_int64: 1, ctypes.c_double: 0.3}
    checked = 0
    for name, res, args in _lib.SIGNATURES:
        if not args or args[0] is not ctypes.c_void_p or name in ("axia_gpu_create",):
            continue
        if not (name.startswith("axia_gpu_") or name.startswith("axia_dofmap_")):
            continue
        call = [defaults.get(a) for a in args]
        r = getattr(lib, name)(*call)
        if res is None:
            assert r is None, name
        elif res is ctypes.c_char_p:
            assert r, name
        elif res is ctypes.c_int64:
            assert r == -1, (name, r)
        else:
            assert r == _lib.ERR_INVALID_ARG, (name, r)
        checked += 1
    assert checked >= 40


def test_struct_layouts_match_header():
    # field order and sizes of the ABI structs (x86-64 and aarch64 share them)
    assert ctypes.sizeof(_lib.Mesh) == 8 * 3 + 4 * 2 + 8 * 4
    assert ctypes.sizeof(_lib.SolveOpts) == 8 + 8 + 4 + 4 + 8 + 4 + 4 + 4 + 4 + 4 + 4 + 4 + 4
    assert ctypes.sizeof(_lib.SolveInfo) == 8 * 4 + 8 * 7 + 8 + 8 + 4 + 4


@pytest.mark.parametrize("model", [meshgen.block_c3d8_pressure(n=5), meshgen.block_c3d20_traction(n=3),
                                   meshgen.patch_c3d20(), meshgen.block_wedge(n=3, nn=6, perturb=0.2),
                                   meshgen.block_wedge(n=2, nn=15, perturb=0.2)],
                         ids=["c3d8", "c3d20", "patch20", "c3d6", "c3d15"])
def test_face_loads_match_oracle(model):
    lib = _lib.load()
    f = np.array(model.cload, dtype=np.float64, copy=True)
    bad = ctypes.c_int64(-1)
    c = np.ascontiguousarray(model.coords)
    cn = np.ascontiguousarray(model.conn, np.int32)
    el = np.ascontiguousarray(model.dload_elem, np.int64)
    fc = np.ascontiguousarray(model.dload_face, np.int32)
    p = np.ascontiguousarray(model.dload_p, np.float64)
    st = lib.axia_face_loads(model.nn, model.n_nodes, c.ctypes.data, cn.ctypes.data, el.shape[0], el.ctypes.data,
                             fc.ctypes.data, p.ctypes.data, f.ctypes.data, ctypes.byref(bad))
    assert st == 0
    ref = O.load_vector(model)
    assert np.abs(f - ref).max() <= 1e-13 * max(1.0, np.abs(ref).max())
    if model.nn in (6, 15):
        # every face of a wedge (extra.rs:184-195, 869-880), bit for bit
        for face in range(1, 6):
            mm = meshgen.block_wedge(n=2, nn=model.nn, perturb=0.2)
            mm.dload_elem = np.arange(mm.conn.shape[0], dtype=np.int64)
            mm.dload_face = np.full(mm.conn.shape[0], face, np.int32)
            mm.dload_p = np.linspace(-3.0, 7.0, mm.conn.shape[0])
            g = np.zeros(3 * mm.n_nodes)
            el = np.ascontiguousarray(mm.dload_elem)
            st = lib.axia_face_loads(mm.nn, mm.n_nodes, np.ascontiguousarray(mm.coords).ctypes.data,
                                     np.ascontiguousarray(mm.conn, np.int32).ctypes.data, el.shape[0],
                                     el.ctypes.data, mm.dload_face.ctypes.data, mm.dload_p.ctypes.data,
                                     g.ctypes.data, ctypes.byref(bad))
            assert st == 0
            np.testing.assert_array_equal(g, O.load_vector(mm))


def test_face_loads_reject_bad_face():
    lib = _lib.load()
    m = meshgen.patch_c3d8()
    f = np.zeros(24)
    el = np.zeros(1, np.int64)
    fc = np.array([7], np.int32)
    p = np.ones(1)
    bad = ctypes.c_int64(-1)
    c = np.ascontiguousarray(m.coords)
    cn = np.ascontiguousarray(m.conn, np.int32)
    st = lib.axia_face_loads(8, 8, c.ctypes.data, cn.ctypes.data, 1, el.ctypes.data, fc.ctypes.data,
                             p.ctypes.data, f.ctypes.data, ctypes.byref(bad))
    assert st == _lib.ERR_INVALID_ARG and bad.value == 0


def test_mesh_sizes_of_the_workloads():
    m = meshgen.cantilever_c3d8()
    assert (m.n_nodes, m.ndof, m.n_free) == (525, 1575, 1500)
    assert np.isclose(m.cload[2::3].sum(), -1000.0)
    coords, conn, lat = meshgen.structured_block(50, 50, 50, 20)
    assert coords.shape[0] == 522801 and conn.shape == (125000, 20)
    coords, conn, lat = meshgen.structured_block(10, 10, 10, 8)
    assert coords.shape[0] == 1331
    # every C3D20 edge node sits halfway between its corner nodes
    coords, conn, _ = meshgen.structured_block(2, 2, 2, 20)
    for e in range(conn.shape[0]):
        x = coords[conn[e]]
        assert np.allclose(x[8], (x[0] + x[1]) / 2) and np.allclose(x[16], (x[0] + x[4]) / 2)


def test_perturbation_keeps_boundary_and_is_seeded():
    a = meshgen.block_c3d8_pressure(n=6)
    b = meshgen.block_c3d8_pressure(n=6)
    assert np.array_equal(a.coords, b.coords)
    _, _, lat = meshgen.structured_block(6, 6, 6, 8)
    bnd = np.any((lat == 0) | (lat == 6), axis=1)
    assert np.array_equal(a.coords[bnd], lat[bnd].astype(float))
    d = np.abs(a.coords[~bnd] - lat[~bnd]).max()
    assert 0 < d <= 0.15


def test_backend_aliases():
    pin = {"FAER": SparseBackend.Faer, "rivrs-sparse": SparseBackend.Rivrs, "intel": SparseBackend.Mkl}
    for s, b in pin.items():  # backend.rs:130-135
        assert parse_sparse_backend(s) == b
    with pytest.raises(BackendError):
        parse_sparse_backend("umfpack")
    assert parse_sparse_backend("gpu") == SparseBackend.Gpu
    assert parse_sparse_backend("--solver=CUDA") == SparseBackend.Gpu
    assert parse_sparse_backend("gpu-mixed") == SparseBackend.GpuMixed
    assert SparseBackend.Gpu.as_str() == "gpu"


def test_backend_selection_and_override(monkeypatch):
    set_sparse_backend(SparseBackend.Auto)
    monkeypatch.setenv("AXIA_SOLVER", "gpu-mixed")
    apply_env_solver()
    assert sparse_backend() == SparseBackend.GpuMixed
    with with_sparse_backend(SparseBackend.Pcg):
        assert sparse_backend() == SparseBackend.Pcg
    assert sparse_backend() == SparseBackend.GpuMixed
    set_sparse_backend(SparseBackend.Auto)
