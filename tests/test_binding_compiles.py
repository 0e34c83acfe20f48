"""The reference-side binding shown in INTEGRATION.md (feMatrixGpu, a subclass
of the operator that routes feMatrix::matVec through the C ABI) compiles
against the reference's own headers and include/dkt_gb300.h.  Runs where the
reference sources are present (the fixture-generation container); skipped
elsewhere."""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("DKT_REFERENCE_DIR", "/root/reference")


def _snippet():
    s = open(os.path.join(REPO, "INTEGRATION.md")).read()
    i = s.index("// FEM/include/feMatrixGpu.h")
    return "#pragma once\n" + s[i:s.index("```", i)]


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "FEM", "include")) or not shutil.which("g++"),
                    reason="reference headers or g++ not available")
def test_fematrix_gpu_binding_compiles(tmp_path):
    (tmp_path / "feMatrixGpu.h").write_text(_snippet())
    (tmp_path / "use.cpp").write_text(
        '#include <mpi.h>\n#include "heatMat.h"\n#include "feMatrixGpu.h"\n'
        "int main(int argc, char **argv) {\n"
        "  MPI_Init(&argc, &argv);\n"
        "  std::vector<ot::TreeNode<unsigned, 3>> tree;\n"
        "  ot::DA<3> *da = nullptr;\n"
        "  feMatrixGpu<HeatEq::HeatMat<3>, 3> A(da, tree, DKT_OP_HEAT);\n"
        "  std::vector<double> x, y;\n"
        "  A.matVec(x.data(), y.data(), 1.0);\n"
        "  return 0;\n}\n")
    inc = [os.path.join(REPO, "oracle", "ref", "shim"), os.path.join(REF, "include"),
           os.path.join(REF, "FEM", "include"), os.path.join(REF, "FEM", "examples", "include"),
           os.path.join(REF, "IO", "vtk", "include"), os.path.join(REF, "array", "include"),
           os.path.join(REPO, "include"), str(tmp_path)]
    cmd = ["g++", "-std=c++14", "-fsyntax-only", "-w", "-DWITH_BLAS_LAPACK", "-DUSE_64BIT_INDICES"]
    cmd += ["-I" + d for d in inc] + [str(tmp_path / "use.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
