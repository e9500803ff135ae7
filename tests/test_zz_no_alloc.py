"""The allocation-free element-stiffness entry point, through the C ABI.

axia_gpu_element_ke_noalloc serves callers that may not allocate GPU memory
(memory owned by another allocator, or loops where an allocation's implicit
synchronization is not acceptable); its only device memory is a fixed array
inside the library.  Its results must equal the context path's
(axia_gpu_element_ke) within the element tolerance of the other tests
(1e-12 of max|Ke|), on consecutive calls that reuse that array.  This file
is collected last so a failure here cannot hide the other tests; it also
passes on its own in a fresh process (the first call sets the array up).
"""
import ctypes

import numpy as np
import pytest

from axia_gpu import GpuContext, _lib, meshgen

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _elements(nn, count, seed):
    rng = np.random.default_rng(seed)
    base = (meshgen.HEX20_XI[:nn].astype(float) + 1) / 2
    out = np.empty((count, nn, 3))
    for k in range(count):
        scale = rng.uniform(0.5, 3.0, 3)
        out[k] = base * scale + rng.uniform(-0.08, 0.08, (nn, 3)) * scale.min() + rng.uniform(-5, 5, 3)
    return out


def _noalloc(xyz, e, nu, reduced=False):
    lib = _lib.load()
    xyz = np.ascontiguousarray(xyz, np.float64)
    n_elem, nn = xyz.shape[0], xyz.shape[1]
    e = np.ascontiguousarray(np.broadcast_to(e, (n_elem,)), np.float64)
    ke = np.zeros((n_elem, 3 * nn, 3 * nn))
    vol = np.zeros(n_elem)
    bad = ctypes.c_int64(-1)
    st = lib.axia_gpu_element_ke_noalloc(nn, int(reduced), n_elem, xyz.ctypes.data, e.ctypes.data, float(nu),
                                         ke.ctypes.data, vol.ctypes.data, ctypes.byref(bad))
    return st, ke, vol, bad.value


@pytest.fixture(scope="module")
def ctx(gpu_ctx):
    return gpu_ctx


@pytest.mark.parametrize("nn,reduced,count", [(8, False, 2048), (20, False, 300), (20, True, 512)])
def test_noalloc_matches_context_path_on_two_calls(ctx, nn, reduced, count):
    for call, seed in enumerate((1, 2)):
        xyz = _elements(nn, count - 7 * call, seed + nn)
        e = np.random.default_rng(seed).uniform(1e3, 2e5, xyz.shape[0])
        st, ke, vol, bad = _noalloc(xyz, e, 0.3, reduced)
        assert st == _lib.OK and bad == -1
        ref, rvol = ctx.element_ke(xyz, e, 0.3, reduced=reduced)
        scale = np.abs(ref).max()
        assert np.abs(ke - ref).max() <= TOL * scale, call
        assert np.abs(vol - rvol).max() <= 1e-13 * np.abs(rvol).max(), call


def test_noalloc_limits_and_errors(ctx):
    st, *_ = _noalloc(_elements(8, 2049, 3), 1.0, 0.3)
    assert st == _lib.ERR_TOO_LARGE
    st, *_ = _noalloc(_elements(20, 513, 3), 1.0, 0.3)
    assert st == _lib.ERR_TOO_LARGE
    xyz = _elements(8, 10, 4)
    xyz[6] = xyz[6][[4, 5, 6, 7, 0, 1, 2, 3]]
    st, ke, vol, bad = _noalloc(xyz, 1.0, 0.3)
    assert st == _lib.ERR_NEG_JACOBIAN and bad == 6
    # the status word is cleared on the next call
    st, ke, vol, bad = _noalloc(_elements(8, 10, 5), 1.0, 0.3)
    assert st == _lib.OK and bad == -1


@pytest.mark.parametrize("nn,reduced", [(8, 1), (8, 2), (20, 2), (20, -1), (4, 0), (10, 0), (6, 0), (15, 0)])
def test_noalloc_rejects_unsupported_kinds(ctx, nn, reduced):
    """Only C3D8, C3D20 and C3D20R: C3D8R / C3D8I and the other kinds are refused, not
    answered with another element's stiffness."""
    xyz = np.zeros((3, nn, 3))
    st, ke, vol, bad = _noalloc(xyz, 1.0, 0.3, reduced)
    assert st == _lib.ERR_INVALID_ARG and bad == -1
    assert not ke.any()
