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


def test_dword_element_stiffness(tmp_path):
    """The double-word closed form of the element kernels (C3D8, C3D20),
    emulated on the host in the kernels' order, against an independent
    long-double B^T D B stiffness: within 1e-13 of max|Ke| (measured about
    3e-14 for C3D8, 8e-14 for C3D20) on distorted elements of edge 1e-3 to 1e3
    up to 100 edges from the origin; the shape derivatives both share pass
    partition of unity and linear completeness."""
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no g++")
    exe = str(tmp_path / "dword_element_check")
    src = os.path.join(HERE, "host", "dword_element_check.cpp")
    subprocess.run([cxx, "-std=c++17", "-O2", "-ffp-contract=off", src, "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
