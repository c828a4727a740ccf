"""The reference's C++ call sequence compiled against include/ahx_ahmed.hpp."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "dropin_sphere.cpp")
LIBDIR = os.path.join(ROOT, "ahmed_gb300")


def _build(tmp_path):
    exe = str(tmp_path / "dropin_sphere")
    subprocess.check_call(["g++", "-O2", "-std=c++14", "-I", os.path.join(ROOT, "include"), SRC,
                           "-L", LIBDIR, "-lahx", "-Wl,-rpath," + LIBDIR, "-o", exe])
    return exe


def test_dropin_compiles_and_builds_trees_on_host(tmp_path):
    exe = _build(tmp_path)
    out = subprocess.run([exe, "2048", "tree-only"], capture_output=True, text=True, check=True)
    assert out.stdout.startswith("leaves ")


@pytest.mark.gpu
def test_dropin_runs_on_gpu(tmp_path):
    exe = _build(tmp_path)
    out = subprocess.run([exe, "2048"], capture_output=True, text=True, timeout=300, cwd=str(tmp_path))
    assert out.returncode == 0, out.stdout + out.stderr
    assert "GMRes ret 0" in out.stdout
    assert "savembls/loadmbls round trip ok" in out.stdout
    assert "symmetric:" in out.stdout
    assert "helmholtz:" in out.stdout
    assert "helmholtz symmetric:" in out.stdout
    assert "helmholtz savembls/loadmbls round trip ok" in out.stdout
    assert "helmholtz agglH:" in out.stdout
    assert "single precision:" in out.stdout


FOREIGN_GENERATOR = r"""
#include "ahx_ahmed.hpp"
using namespace ahx_ahmed;
struct MyGen {  // a program's own MATGEN_T (Include/matgen_omp.h:27-33)
  double geth() const { return 1.0; }
  void cmpbl(unsigned, unsigned, unsigned, unsigned, double*) const {}
  double scale(unsigned, unsigned, unsigned, unsigned) const { return 1.0; }
};
void f(blcluster* bl, mblock<double>** A) { MyGen g; matgenGeH_omp(g, 1u, bl, 1e-6, 100u, A); }
"""

FOREIGN_COMPLEX_GENERATOR = r"""
#include "ahx_ahmed.hpp"
using namespace ahx_ahmed;
void f(blcluster* bl, mblock<dcomp>** A) { LaplaceGenerator g{1.0}; matgenGeH_omp(g, 1u, bl, 1e-6, 100u, A); }
"""

FOREIGN_MATRIX = r"""
#include "ahx_ahmed.hpp"
using namespace ahx_ahmed;
struct MyMat : Matrix<double> {  // a program's own operator with a preconditioner
  MyMat() : Matrix<double>(4, 4) {}
  void amux(double, double*, double*) const override {}
  void precond_apply(double*) const override {}
};
unsigned f(double* b, double* x) { MyMat A; double e = 1e-8; unsigned n = 10; return %s; }
"""


def _compile(tmp_path, src, name):
    path = tmp_path / (name + ".cpp")
    path.write_text(src)
    return subprocess.run(["g++", "-std=c++14", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), str(path)],
                          capture_output=True, text=True)


@pytest.mark.parametrize("src,msg", [(FOREIGN_GENERATOR, "LaplaceGenerator"),
                                     (FOREIGN_COMPLEX_GENERATOR, "HelmholtzGenerator")])
def test_foreign_generator_does_not_compile(tmp_path, src, msg):
    """A MATGEN_T that is not one of the library's GPU generators is refused at
    compile time (its cmpbl/scale would not be evaluated)."""
    r = _compile(tmp_path, src, "gen")
    assert r.returncode != 0
    assert msg in r.stderr and "static assertion" in r.stderr


@pytest.mark.parametrize("call", ["GMRes(A, b, x, e, 30u, n)", "CG(A, b, x, e, n)"])
def test_solver_on_foreign_matrix_does_not_compile(tmp_path, call):
    """GMRes / CG take the library's operators only; a program's own Matrix<T> (whose
    precond_apply these solvers would not apply) is refused at compile time."""
    r = _compile(tmp_path, FOREIGN_MATRIX % call, "mat")
    assert r.returncode != 0
    assert "deleted" in r.stderr


def test_library_operators_compile(tmp_path):
    src = r"""
#include "ahx_ahmed.hpp"
using namespace ahx_ahmed;
unsigned f(blcluster* bl, double* b, double* x) {
  HMatrixOperator A(bl); double e = 1e-8; unsigned n = 10;
  return GMRes(A, b, x, e, 30u, n) + CG(A, b, x, e, n);
}
"""
    r = _compile(tmp_path, src, "ok")
    assert r.returncode == 0, r.stderr
