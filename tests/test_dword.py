"""Host check of the double-word (FP32 pair) primitives that the element
stiffness kernel runs on the FP32 pipe (axia-fem_gb300/csrc/dword.cuh):
TwoSum and TwoProduct exact, FP32 -> FP64 re-encoding exact for every class
of number, round trips within 2^-48, products / quotients / compensated dot
products within small multiples of 2^-48.  Compiled with g++ -ffp-contract=off
(the device code uses explicit round-to-nearest intrinsics)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_dword_primitives(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no g++")
    exe = str(tmp_path / "dword_check")
    src = os.path.join(HERE, "host", "dword_check.cpp")
    subprocess.run([cxx, "-std=c++17", "-O2", "-ffp-contract=off", src, "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
