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


ADAPTERS_TU = r"""
// every adapter of include/pdg/pdelab.hh, compiled and linked (not run here)
#include <vector>
#include "pdg/pdelab.hh"

int drive(int n) {
  pdg::Config cfg(3, 2, n, n, n);
  pdg::GridOperator go(cfg);
  const long nd = go.size(), nc = go.cells();
  std::vector<double> x(nd, 0.0), y(nd, 0.0), z(nd, 0.0), g(nc, 0.0);
  go.setPermeability(std::vector<double>(nc, 0.0), true);
  go.setReaction(std::vector<double>(nc, 1.0));
  go.setVelocityModes({1, 0, 0, 0.3, 0, 1, 0});
  go.setNonlinearity({0.0, 0.0, 1.0});
  go.setNonlinearity({});
  go.setF64Arithmetic(PDG_F64_NATIVE);
  const std::vector<double> &cx = x;   // read-only inputs bind to const vectors
  go.residual(cx, y);
  go.jacobian_apply(cx, y);
  go.jacobian_apply(x, z, y);
  go.jacobian_apply_transpose(x, y);
  go.mass_apply(x, y);
  pdg::GridOperator::BCRSMatrix A;
  go.jacobian(A);
  pdg::OnTheFlyOperator op(go);
  op.apply(x, y);
  op.applyscaleadd(-1.0, x, y);
  op.setLinearizationPoint(x);
  pdg::GridOperatorPreconditioner prec(go);
  prec.pre(x, y);
  prec.apply(x, y);
  prec.setLinearizationPoint(x);
  prec.post(x);
  pdg::ISTLBackend_SEQ_MatrixFree_Base ls(go, PDG_BICGSTAB);
  ls.setMixedPrecision(true, 1e-4);
  ls.apply(z, y, 1e-10);
  double nrm = ls.norm(y) + ls.result().iterations;
  pdg::StationaryLinearProblemSolver slp(go, ls, x, 1e-10);
  slp.apply();
  pdg::NewtonMethod newton(go, ls);
  newton.setReduction(1e-10);
  newton.setAbsoluteLimit(1e-12);
  newton.setMinLinearReduction(1e-3);
  newton.setFixedLinearReduction(false);
  newton.setMaxIterations(20);
  newton.setForceIteration(false);
  newton.setLineSearch(true);
  newton.setLineSearchMaxIterations(10);
  newton.setLineSearchDampingFactor(0.5);
  newton.setLineSearchAcceptBest(false);
  newton.setVerbosityLevel(0);
  newton.apply(x);
  nrm += newton.result().iterations;
  pdg::OneStepMethod osm(go, ls, PDG_ONESTEP_ALEXANDER2);
  osm.setMethod(PDG_ONESTEP_THETA, 0.5);
  nrm += osm.apply(0.0, 0.1, x, z) + osm.result().stages;
  pdg::Adjoint adj(go, ls);
  adj.solve(y, z, 1e-10);
  adj.gradLogK(cx, cx, g);
  adj.gradLogK(x, z, g);
  adj.gradSource(z, g);
  return (int)(nrm + adj.result().iterations + A.rows);
}

int main(int argc, char **) { return argc > 5 ? drive(argc) : 0; }
"""


def test_cpp_adapters_compile_and_link(tmp_path):
    # every C++ adapter against the C ABI, compiled with warnings as errors and
    # linked against libpdg.so; the program is not run (no GPU needed)
    import __graft_entry__
    __graft_entry__.build()
    src = tmp_path / "adapters.cc"
    src.write_text(ADAPTERS_TU)
    exe = tmp_path / "adapters"
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I",
           os.path.join(ROOT, "include"), str(src), "-L", os.path.join(PKG, "_build"), "-lpdg",
           "-Wl,-rpath," + os.path.join(PKG, "_build"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert exe.exists()


EXE2 = os.path.join(PKG, "_build", "adjoint_newton_onestep")


def _build_adapters_driver():
    import __graft_entry__
    __graft_entry__.build()
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I",
           os.path.join(ROOT, "include"), os.path.join(PKG, "examples", "adjoint_newton_onestep.cc"),
           "-L", os.path.join(PKG, "_build"), "-lpdg",
           "-Wl,-rpath," + os.path.join(PKG, "_build"), "-o", EXE2]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_cpp_adjoint_newton_onestep_builds():
    _build_adapters_driver()
    assert os.path.exists(EXE2)


@pytest.mark.gpu
def test_cpp_adjoint_newton_onestep():
    # the adjoint, BCRS export, Newton and one-step adapters from C++ on the
    # GPU, each against its own identity (central differences, A x = J x,
    # R(u) = 0, the implicit Euler equation)
    _build_adapters_driver()
    r = subprocess.run([EXE2], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["adjoint_fd_rel_logK"] < 1e-5 and out["adjoint_fd_rel_source"] < 1e-5
    assert out["bcrs_rel"] < 1e-12 and out["bcrs_transpose_rel"] < 1e-12
    assert out["nipg_asymmetry"] > 1e-6
    assert out["newton_converged"] == 1 and out["newton_residual_rel"] < 1e-9
    assert out["implicit_euler_rel"] < 1e-10
