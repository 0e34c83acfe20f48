"""The reference-side binding include/feMatrixGpu.h (feMatrixGpu, a subclass
of the operator that routes feMatrix::matVec and HeatMat::cgSolve through the
C ABI) compiles against the reference's own headers and include/dkt_gb300.h,
in both curve builds.  Runs where the reference sources are present (the
fixture-generation container); skipped elsewhere."""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("DKT_REFERENCE_DIR", os.path.join(os.path.dirname(REPO), "reference"))


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "FEM", "include")) or not shutil.which("g++"),
                    reason="reference headers or g++ not available")
@pytest.mark.parametrize("curve", ["", "-DHILBERT_ORDERING"], ids=["morton", "hilbert"])
def test_fematrix_gpu_binding_compiles(tmp_path, curve):
    (tmp_path / "use.cpp").write_text(
        '#include <mpi.h>\n#include "heatMat.h"\n#include "feMatrixGpu.h"\n'
        "int main(int argc, char **argv) {\n"
        "  MPI_Init(&argc, &argv);\n"
        "  std::vector<ot::TreeNode<unsigned, 3>> tree;\n"
        "  ot::DA<3> *da = nullptr;\n"
        "  feMatrixGpu<HeatEq::HeatMat<3>, 3> A(da, tree, DKT_OP_HEAT);\n"
        "  std::vector<double> x, y;\n"
        "  A.matVec(x.data(), y.data(), 1.0);\n"
        "  double tol = 1e-10;\n"
        "  return A.cgSolve(x.data(), y.data(), 100, tol);\n}\n")
    inc = [os.path.join(REPO, "oracle", "ref", "shim"), os.path.join(REF, "include"),
           os.path.join(REF, "FEM", "include"), os.path.join(REF, "FEM", "examples", "include"),
           os.path.join(REF, "IO", "vtk", "include"), os.path.join(REF, "array", "include"),
           os.path.join(REPO, "include")]
    cmd = ["g++", "-std=c++14", "-fsyntax-only", "-w", "-DWITH_BLAS_LAPACK", "-DUSE_64BIT_INDICES"]
    cmd += [curve] if curve else []
    cmd += ["-I" + d for d in inc] + [str(tmp_path / "use.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
