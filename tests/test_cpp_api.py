"""The C++ stand-ins of the reference API (include/dgcu.hpp): the
dgEulerFoam-style example compiles against the C ABI here, and on a GPU the
solveEquation-driven stage loop reproduces the device integrator."""
import os
import subprocess

import pytest

from conftest import ROOT

EXAMPLE = os.path.join(ROOT, "hopefoam_gb300", "examples", "dgEulerFoam.cpp")
CUB = os.path.join(ROOT, "hopefoam_gb300", "data", "tri_cubature.txt")


def _compile(tmp_path):
    from hopefoam_gb300 import build

    lib = build.build()
    exe = str(tmp_path / "dgEulerFoam")
    cmd = ["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), EXAMPLE, "-o", exe,
           "-L" + os.path.dirname(lib), "-ldgcu", "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_example_compiles(tmp_path):
    _compile(tmp_path)


@pytest.mark.gpu
def test_example_runs_on_gpu(tmp_path, gpu_lib):
    exe = _compile(tmp_path)
    r = subprocess.run([exe, CUB, "12", "3", "5"], capture_output=True, text=True, timeout=300)
    print(r.stdout, r.stderr)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "solveEquation-vs-integrator" in r.stdout
