"""The C++ adapters (include/pdg/pdelab.hh) build a PDELab-shaped driver
(examples/matrix_free_linear.cc) against libpdg.so; on a GPU it reproduces
the reference test's criterion (L2 error^2 < 1e-6)."""
import json
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "dune-pdelab_gb300")
EXE = os.path.join(PKG, "_build", "matrix_free_linear")


def _build():
    import __graft_entry__
    __graft_entry__.build()
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
           os.path.join(PKG, "examples", "matrix_free_linear.cc"),
           "-L", os.path.join(PKG, "_build"), "-lpdg",
           "-Wl,-rpath," + os.path.join(PKG, "_build"), "-o", EXE]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_cpp_driver_builds():
    _build()
    assert os.path.exists(EXE)


@pytest.mark.gpu
def test_cpp_driver_matrix_free_linear():
    _build()
    r = subprocess.run([EXE, "16"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["converged"] == 1 and out["l2errorsquared"] < 1e-6
