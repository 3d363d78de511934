"""The Eigen backend header (include/eigen_gb300/LLT_GB300.h) under Eigen's own unit tests.

Eigen's test/cholesky.cpp and test/inplace_decomposition.cpp are compiled where they lie (they are
never copied) with the backend header placed right after Eigen's test harness, and linked against
a test double of libgbllt (tests/eigen/fake_gbllt.c) that forwards each C-ABI call to the oracle
and counts it.  The tests' own assertions (VERIFY_IS_APPROX at 1e-6 / 1e-3, the NumericalIssue
checks, the in-place semantics of LLT<Ref<MatrixXd>>) must all hold, and the call counts prove
the specialisations were selected.  This checks the header's plumbing (layout, uplo, info mapping,
leading dimensions, the solve hooks) on the CPU; the GPU kernels behind the C ABI are checked by
the gpu-marked tests.  Needs the Eigen sources ($EIGEN_REF, or the tree the oracle's `ref` build
used) and g++.
"""
import os
import re
import shutil
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "oracle"))
import oracle as _oracle  # noqa: E402

EIGEN = _oracle.eigen_src()
pytestmark = pytest.mark.skipif(EIGEN is None or not (EIGEN / "Eigen" / "Cholesky").exists() or
                                shutil.which("g++") is None,
                                reason="Eigen sources or g++ not available")


@pytest.fixture(scope="module")
def objs(tmp_path_factory):
    d = tmp_path_factory.mktemp("eigen_backend")
    fake = d / "fake.o"
    orc = d / "oracle.o"
    subprocess.run(["gcc", "-O2", "-fopenmp", "-c", str(ROOT / "tests/eigen/fake_gbllt.c"), "-o", str(fake)], check=True)
    subprocess.run(["gcc", "-O2", "-fopenmp", "-c", str(ROOT / "oracle/llt_oracle.c"), "-o", str(orc)], check=True)
    return d, [str(fake), str(orc)]


def _build_and_run(objs, test_name):
    d, links = objs
    exe = d / f"{test_name}_gb300"
    cmd = ["g++", "-O1", "-std=c++14", "-w",
           "-I", str(ROOT / "tests/eigen/shim"), "-I-",      # the tests' #include "main.h" -> shim
           "-I", str(EIGEN / "test"), "-I", str(EIGEN), "-I", str(EIGEN / "Eigen"),
           "-I", str(EIGEN / "Eigen/src/Core"), "-I", str(EIGEN / "Eigen/src/plugins"),
           "-I", str(ROOT / "include"),
           f'-DEIGEN_TEST_HARNESS="{EIGEN / "test" / "main.h"}"', "-DEIGEN_TEST_MAX_SIZE=320",
           "-DEIGEN_TEST_PART_ALL=1", str(EIGEN / "test" / f"{test_name}.cpp"), *links, "-o", str(exe),
           "-lm", "-fopenmp"]
    subprocess.run(cmd, check=True, capture_output=True)
    res = subprocess.run([str(exe), "r3", "s1234"], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-2000:]
    m = re.search(r"fake_gbllt calls: dpotrf=(\d+) spotrf=(\d+) dpotrs=(\d+) spotrs=(\d+) dpocon=(\d+) "
                  r"spocon=(\d+) drankupd=(\d+) srankupd=(\d+) dldlt=(\d+) sldlt=(\d+) dldlts=(\d+) "
                  r"sldlts=(\d+) dtrsm=(\d+) strsm=(\d+)", res.stderr)
    assert m, res.stderr[-2000:]
    return [int(v) for v in m.groups()]


def test_eigen_cholesky_suite_through_backend(objs):
    dpotrf, spotrf, dpotrs, _, dpocon, _, drankupd, srankupd, dldlt, _, dldlts, _, _, _ = _build_and_run(objs,
                                                                                                       "cholesky")
    # MatrixXd factorisations, solves, condition estimates and rank updates, and fixed-size float
    # factorisations and rank updates, went through the C ABI (the rcond checks of
    # test/cholesky.cpp:94-115 ran on gbllt_dpocon, the rankUpdate checks of :44-56 on gbllt_?rank_update)
    assert dpotrf > 0 and dpotrs > 0 and spotrf > 0 and dpocon > 0 and drankupd > 0 and srankupd > 0
    # LDLT<MatrixXd> factorisations (including the definiteness and failure cases of
    # test/cholesky.cpp:358-469) and solves went through gbllt_dldlt / gbllt_dldlt_solve
    assert dldlt > 0 and dldlts > 0


def test_eigen_inplace_decomposition_through_backend(objs):
    counts = _build_and_run(objs, "inplace_decomposition")
    assert counts[0] > 0  # LLT<Ref<MatrixXd>>
    assert counts[8] > 0  # LDLT<Ref<MatrixXd>> (test/inplace_decomposition.cpp runs both)


def test_eigen_trsolve_suite_through_backend(objs):
    # test/product_trsolve.cpp: every triangular view (Lower/Upper/UnitLower/UnitUpper, either storage
    # order, on the left and on the right, solveInPlace and solve) of float and double matrices up to
    # the test's maximum size, checked by the test's own VERIFY_IS_APPROX; the complex cases stay on
    # Eigen's CPU code
    counts = _build_and_run(objs, "product_trsolve")
    assert counts[12] > 0 and counts[13] > 0  # gbllt_dtrsm, gbllt_strsm


def test_llt_solve_in_place_through_backend(objs, tmp_path):
    # LLT::solveInPlace (LLT.h:514-522) bypasses Solve<> and calls the two triangular views: with the
    # backend its triangular solves go through gbllt_dtrsm (a matrix of right-hand sides) and the
    # vector hook (one right-hand side); the result matches llt.solve(b)
    d, links = objs
    src = tmp_path / "llt_solve_in_place.cpp"
    src.write_text(r"""
#include <Eigen/Cholesky>
#include <cstdio>
int main() {
  using namespace Eigen;
  const int n = 97;
  MatrixXd g = MatrixXd::Random(n, n);
  MatrixXd a = g * g.transpose() / n + MatrixXd::Identity(n, n);
  LLT<MatrixXd> llt(a);
  MatrixXd b = MatrixXd::Random(n, 5), x = b;
  llt.solveInPlace(x);
  VectorXd v = VectorXd::Random(n), y = v;
  llt.solveInPlace(y);
  LLT<MatrixXd, Upper> lltu(a);
  MatrixXd xu = b;
  lltu.solveInPlace(xu);
  const double e1 = (a * x - b).norm() / b.norm(), e2 = (a * y - v).norm() / v.norm();
  const double e3 = (a * xu - b).norm() / b.norm();
  std::printf("%g %g %g\n", e1, e2, e3);
  return (e1 < 1e-12 && e2 < 1e-12 && e3 < 1e-12) ? 0 : 1;
}
""")
    exe = d / "llt_solve_in_place"
    subprocess.run(["g++", "-O1", "-std=c++14", "-w", "-I", str(EIGEN), "-I", str(ROOT / "include"),
                    "-DEIGEN_USE_GB300", "-include", "eigen_gb300/LLT_GB300.h", str(src), *links, "-o", str(exe),
                    "-lm", "-fopenmp"], check=True, capture_output=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stdout + res.stderr
    m = re.search(r"dtrsm=(\d+)", res.stderr)
    assert m and int(m.group(1)) >= 6  # two triangular solves per solveInPlace, three calls
