"""GPU element stiffness (axia_gpu_element_ke) against the oracle's restated
hex8_stiffness / hex20_stiffness (solver/src/elem.rs:194-219,
solver/src/quadratic.rs:122-146).  FP64 tolerance: 1e-12 relative to max|Ke|."""
import json
import os

import numpy as np
import pytest

from axia_gpu import _lib, meshgen
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))["vectors"]
TOL = 1e-12


def _rand_elems(nn, count, seed):
    rng = np.random.default_rng(seed)
    xi = meshgen.HEX20_XI[:nn].astype(float)
    base = (xi + 1) / 2
    out = np.empty((count, nn, 3))
    for k in range(count):
        scale = rng.uniform(0.5, 3.0, 3)
        out[k] = base * scale + rng.uniform(-0.08, 0.08, (nn, 3)) * scale.min() + rng.uniform(-5, 5, 3)
    return out


@pytest.mark.parametrize("nn,reduced", [(8, False), (20, False), (20, True)])
def test_element_ke_matches_oracle(gpu_ctx, nn, reduced):
    xyz = _rand_elems(nn, 37, seed=nn + reduced)
    e = np.random.default_rng(3).uniform(1e3, 2e5, xyz.shape[0])
    ke, vol = gpu_ctx.element_ke(xyz, e, 0.3, reduced=reduced)
    for k in range(xyz.shape[0]):
        ref, rvol = O.element_ke(xyz[k], e[k], 0.3, reduced=reduced)
        scale = np.abs(ref).max()
        assert np.abs(ke[k] - ref).max() <= TOL * scale, k
        assert abs(vol[k] - rvol) <= 1e-13 * rvol


def test_element_ke_golden_vectors(gpu_ctx):
    for key, red in (("hex8_distorted", False), ("hex20_distorted", False)):
        g = GOLD[key]
        ke, vol = gpu_ctx.element_ke(np.array(g["xyz"]), g["e"], g["nu"], reduced=red)
        ref = np.array(g["ke"]).reshape(ke.shape[1:])
        assert np.abs(ke[0] - ref).max() <= TOL * np.abs(ref).max()
    g = GOLD["hex20_distorted"]
    ke, _ = gpu_ctx.element_ke(np.array(g["xyz"]), g["e"], g["nu"], reduced=True)
    ref = np.array(GOLD["hex20r_distorted"]["ke"]).reshape(60, 60)
    assert np.abs(ke[0] - ref).max() <= TOL * np.abs(ref).max()


def test_element_errors_report_first_bad_element(gpu_ctx):
    xyz = _rand_elems(8, 10, seed=5)
    bad = xyz.copy()
    bad[7] = bad[7][[4, 5, 6, 7, 0, 1, 2, 3]]   # inverted: det J < 0
    bad[3] = bad[3][[4, 5, 6, 7, 0, 1, 2, 3]]
    with pytest.raises(_lib.AxiaError) as e:
        gpu_ctx.element_ke(bad, 1.0, 0.3)
    assert e.value.code == _lib.ERR_NEG_JACOBIAN and e.value.bad_index == 3
    flat = xyz.copy()
    flat[2, :, 2] = 0.0
    with pytest.raises(_lib.AxiaError) as e:
        gpu_ctx.element_ke(flat, 1.0, 0.3)
    assert e.value.code == _lib.ERR_SINGULAR_JACOBIAN and e.value.bad_index == 2
    with pytest.raises(_lib.AxiaError) as e:
        gpu_ctx.element_ke(xyz, 1.0, 0.5)
    assert e.value.code == _lib.ERR_MATERIAL
    ee = np.ones(10)
    ee[6] = -1.0
    with pytest.raises(_lib.AxiaError) as e:
        gpu_ctx.element_ke(xyz, ee, 0.3)
    assert e.value.code == _lib.ERR_MATERIAL and e.value.bad_index == 6
    nan = xyz.copy()
    nan[9, 3, 1] = np.nan
    with pytest.raises(_lib.AxiaError) as e:
        gpu_ctx.element_ke(nan, 1.0, 0.3)
    assert e.value.code == _lib.ERR_NONFINITE and e.value.bad_index == 9
    # the context stays usable after element errors
    ke, _ = gpu_ctx.element_ke(xyz, 1.0, 0.3)
    assert np.isfinite(ke).all()


def test_element_ke_empty_and_large_batch(gpu_ctx):
    ke, vol = gpu_ctx.element_ke(np.zeros((0, 8, 3)), np.zeros(0), 0.3)
    assert ke.shape == (0, 24, 24)
    xyz = _rand_elems(8, 5000, seed=9)
    ke, vol = gpu_ctx.element_ke(xyz, 1.0, 0.25)
    for k in (0, 1234, 4999):
        ref, _ = O.element_ke(xyz[k], 1.0, 0.25)
        assert np.abs(ke[k] - ref).max() <= TOL * np.abs(ref).max()


def _placed_elems(nn, count, seed, offset, size, amp):
    """Elements of edge ~size, corners/midsides moved by up to amp*size, placed up to offset from the origin."""
    rng = np.random.default_rng(seed)
    base = (meshgen.HEX20_XI[:nn].astype(float) + 1) / 2
    out = np.empty((count, nn, 3))
    for k in range(count):
        scale = size * rng.uniform(0.5, 2.0, 3)
        out[k] = base * scale + rng.uniform(-amp, amp, (nn, 3)) * scale.min() + rng.uniform(-offset, offset, 3)
    return out


@pytest.mark.parametrize("arith", [_lib.ELEMENT_DWORD, _lib.ELEMENT_FP64])
@pytest.mark.parametrize("nn,reduced", [(8, False), (20, False), (20, True)])
def test_element_arith_matches_oracle_across_sizes_and_offsets(gpu_ctx, arith, nn, reduced):
    """Both element arithmetics against the oracle at 1e-12 of max|Ke|: element
    edges from 1e-3 to 1e3, placed up to 100 edges from the origin.  The
    double-word form works on coordinates relative to the element's first node,
    scaled by a power of two, so size and placement cost it no accuracy."""
    gpu_ctx.set_element_arith(arith)
    try:
        for size, offset in ((1e-3, 0.0), (1.0, 100.0), (1e3, 5e3), (0.05, 2.0)):
            xyz = _placed_elems(nn, 24, seed=nn + 7 * reduced, offset=offset, size=size, amp=0.08)
            e = np.random.default_rng(5).uniform(1e3, 2e11, xyz.shape[0])
            ke, vol = gpu_ctx.element_ke(xyz, e, 0.3, reduced=reduced)
            for k in range(xyz.shape[0]):
                ref, rvol = O.element_ke(xyz[k], e[k], 0.3, reduced=reduced)
                assert np.abs(ke[k] - ref).max() <= TOL * np.abs(ref).max(), (size, offset, k)
                assert abs(vol[k] - rvol) <= 1e-12 * rvol, (size, offset, k)
    finally:
        gpu_ctx.set_element_arith(_lib.ELEMENT_DWORD)


@pytest.mark.parametrize("nn,reduced", [(8, False), (20, False), (20, True)])
def test_element_dword_close_to_fp64(gpu_ctx, nn, reduced):
    """The double-word Ke (node-pair kernel for C3D20 / C3D20R) differs from the
    FP64 kernel's by a few 1e-14 of max|Ke| on moderately distorted elements,
    and is exactly symmetric like it."""
    xyz = _rand_elems(nn, 500, seed=31 + nn + reduced)
    ke_dw, vol_dw = gpu_ctx.element_ke(xyz, 2e5, 0.3, reduced=reduced)
    gpu_ctx.set_element_arith(_lib.ELEMENT_FP64)
    try:
        ke64, vol64 = gpu_ctx.element_ke(xyz, 2e5, 0.3, reduced=reduced)
    finally:
        gpu_ctx.set_element_arith(_lib.ELEMENT_DWORD)
    worst = max(np.abs(ke_dw[k] - ke64[k]).max() / np.abs(ke64[k]).max() for k in range(xyz.shape[0]))
    assert worst <= 1e-13, worst
    assert all(np.array_equal(ke_dw[k], ke_dw[k].T) for k in range(xyz.shape[0]))
    assert np.abs(vol_dw - vol64).max() <= 1e-13 * np.abs(vol64).max()
    with pytest.raises(_lib.AxiaError) as e:
        gpu_ctx.set_element_arith(2)
    assert e.value.code == _lib.ERR_INVALID_ARG
