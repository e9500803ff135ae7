"""Writes tests/golden/golden.json.

Two kinds of content:
  * "pins": the known answers the reference's own tests assert for this path
    (closed-form scalars; the reference stores no displacement vectors), each
    with the file:line of the assertion in larsmei/axia-fem.
  * "vectors": small regression vectors produced by the CPU oracle
    (oracle/axia_oracle.cpp) here, so the oracle can be checked on any machine
    against the same numbers and the GPU tests have fixed expected values.

Run from the repository root:  python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "axia-fem_gb300"))

from axia_gpu import meshgen  # noqa: E402
from oracle import oracle as O  # noqa: E402

PINS = {
    "patch_c3d8_mean_ux": {"value": 0.01, "tol": 1e-6, "nodes_1based": [2, 3, 6, 7],
                           "source": "solver/src/lib.rs:429-439 (patch_test_c3d8)"},
    "patch_c3d8_backends_agree_ux": {"value": 0.01, "tol": 1e-6,
                                     "source": "solver/src/lib.rs:464-496 (sparse_backends_agree_on_c3d8_patch)"},
    "patch_c3d20_mean_ux": {"value": -0.01, "tol": 1e-5, "nodes_1based": [2, 3, 6, 7],
                            "source": "solver/src/lib.rs:751-763 (patch_test_c3d20)"},
    "patch_c3d8_mean_sxx": {"value": 210.0, "tol": 1e-3,
                            "source": "solver/src/lib.rs:440-446 (patch_test_c3d8: mean nodal sxx, vm > 0)"},
    "patch_c3d20_mean_sxx": {"value": -210.0, "tol": 1.0,
                             "source": "solver/src/lib.rs:764-772 (patch_test_c3d20: mean nodal sxx)"},
    "le10_c3d20_syy_D": {"value": -5.51, "tol": 0.005, "target": -5.38, "target_rel_tol": 0.05,
                         "fixture": "le10_c3d20.json",
                         "source": "solver/src/nafems.rs:49-67 (nafems_le10_thick_plate, target -5.38 within 5 %); "
                                   "examples/nafems/README.md:13 (the reference's result -5.51)"},
    "le10_c3d20_fine_syy_D": {"value": -5.50, "tol": 0.005, "target": -5.38, "target_rel_tol": 0.03,
                              "fixture": "le10_c3d20_fine.json",
                              "source": "solver/src/nafems.rs:70-88 (refined, target within 3 %); "
                                        "examples/nafems/README.md:14 (the reference's result -5.50)"},
    "hex20_partition_of_unity": {"value": 1.0, "tol": 1e-12,
                                 "source": "solver/src/quadratic.rs:890-894 (hex20_partition)"},
    "quad8_partition_of_unity": {"value": 1.0, "tol": 1e-12,
                                 "source": "solver/src/quadratic.rs:864-887 (quad8_partition_and_jac)"},
    "backend_aliases": {"FAER": "faer", "rivrs-sparse": "rivrs", "intel": "mkl", "umfpack": None,
                        "source": "solver/src/backend.rs:130-135 (parse_aliases)"},
    "residual_ok": {"rule": "||Kx-b|| <= 1e-8 max(||b||,1) + 1e-10",
                    "source": "solver/src/sparse_native.rs:1572-1578"},
    "pcg_defaults": {"tol": 1e-8, "max_iter": "max(4n, 200)", "source": "solver/src/linalg.rs:363, 375-376"},
}


def distorted_hex8(seed=7):
    rng = np.random.default_rng(seed)
    base = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float)
    return base * np.array([2.0, 1.5, 1.0]) + rng.uniform(-0.15, 0.15, base.shape)


def distorted_hex20(seed=11):
    rng = np.random.default_rng(seed)
    xi = meshgen.HEX20_XI.astype(float)
    base = (xi + 1.0) / 2.0 * np.array([1.0, 2.0, 1.5])
    return base + rng.uniform(-0.08, 0.08, base.shape)


def main():
    out = {"pins": PINS, "vectors": {}}
    v = out["vectors"]
    ke, vol = O.element_ke(distorted_hex8(), 210000.0, 0.3)
    v["hex8_distorted"] = {"xyz": distorted_hex8().tolist(), "e": 210000.0, "nu": 0.3, "ke": ke.ravel().tolist(),
                           "vol": vol}
    ke, vol = O.element_ke(distorted_hex20(), 70000.0, 0.33)
    v["hex20_distorted"] = {"xyz": distorted_hex20().tolist(), "e": 70000.0, "nu": 0.33, "ke": ke.ravel().tolist(),
                            "vol": vol}
    ke, vol = O.element_ke(distorted_hex20(), 70000.0, 0.33, reduced=True)
    v["hex20r_distorted"] = {"ke": ke.ravel().tolist(), "vol": vol}
    m = meshgen.cantilever_c3d8()
    r = O.solve_static(m, solver=O.SOLVER_CHOLESKY)
    v["cantilever_20x4x4"] = {"n_free": r.n_free, "nnz_kff": r.nnz, "tip_uz_min": float(r.u[2::3].min()),
                              "u": r.u.tolist(), "solver": "oracle dense Cholesky (linalg.rs:78-117)"}
    stress, vm = O.nodal_stress(m, r.u)
    rf = O.reactions(m, r.u, r.f)
    v["cantilever_20x4x4"].update({"vm": vm.tolist(), "sxx": stress[:, 0].tolist(), "rf": rf.tolist()})
    fe = O.face_pressure(distorted_hex8(), 4, 1.0)
    v["hex8_face_p4"] = {"fe": fe.tolist()}
    fe = O.face_pressure(distorted_hex20(), 2, 1.0)
    v["hex20_face_p2"] = {"fe": fe.tolist()}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")
    with open(path, "w") as fh:
        json.dump(out, fh, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()
