"""bench.py's CPU pieces on a small block: the reference arm's JSON line (the
CPU restatement of the reference's path, timed with every host thread) and
the full-size accuracy check (the oracle's element-by-element residual),
which must vanish for the oracle's own solution and flag a wrong one."""
import argparse
import importlib.util
import json
import os

import numpy as np

from axia_gpu import meshgen
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_reference_arm_line(monkeypatch, capsys):
    bench = _bench()
    monkeypatch.setattr(bench, "CPU_SAMPLE_N", 6)
    monkeypatch.delenv("RANK", raising=False)
    bench.run_reference(argparse.Namespace(steps=1, warmup=3, gpus=1))
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["unit"] == "MDOF/s"
    assert line["value"] > 0 and line["higher_is_better"] is True and line["steps"] == 1 and line["warmup"] == 3
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["cpu_baseline"]["cores"] >= 1 and "6^3" in line["cpu_baseline"]["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": "MDOF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_print_nothing(monkeypatch, capsys):
    bench = _bench()
    monkeypatch.setenv("RANK", "1")
    bench.run_reference(argparse.Namespace(steps=1, warmup=3, gpus=2))
    assert capsys.readouterr().out == ""


def test_oracle_residual_check():
    bench = _bench()
    m = meshgen.block_c3d8_pressure(n=5)
    f = O.load_vector(m)
    r = O.solve_static(m, solver=O.SOLVER_PCG, tol=1e-13, f=f)
    u = np.asarray(r.u, dtype=np.float64)
    bad = u.copy()
    bad[np.argmax(np.abs(u))] *= 1.01
    out = bench.oracle_residuals(m, {"oracle": u, "perturbed": bad}, f)
    res = out["rel_residual_free"]
    assert res["oracle"] <= 2e-13, res
    assert res["perturbed"] > 1e-4, res
