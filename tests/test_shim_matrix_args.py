"""The C++ shim's Eigen-style signatures, checked on the CPU with mock
matrix types (no Eigen in this build environment, no device calls).

The reference's C++ API takes column-major Eigen::MatrixXf poses and images
and writes Eigen::Ref<MRow> outputs (include/mrfmap/GVDBInference.h:87-102,
include/mrfmap/GVDBMapLikelihoodEstimator.h:97-117).  The shim headers
overload every such method for any matrix type with rows(), cols() and
m(i, j): tests/cpp/overloads_compile.cpp makes the reference's calls with
mocks (compiled to an object: every call resolves, the pointer forms still
resolve to themselves), tests/cpp/matrix_args_run.cpp runs the layout
conversions."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CPP = os.path.join(ROOT, "tests", "cpp")
CXX = os.environ.get("CXX") or shutil.which("g++")

pytestmark = pytest.mark.skipif(CXX is None, reason="no C++ compiler")


def _cxx(*args):
    r = subprocess.run([CXX, "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), "-I", CPP,
                        *args], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_reference_style_calls_resolve(tmp_path):
    _cxx("-c", os.path.join(CPP, "overloads_compile.cpp"), "-o", str(tmp_path / "o.o"))


def test_matrix_layouts(tmp_path):
    exe = tmp_path / "matrix_args"
    _cxx(os.path.join(CPP, "matrix_args_run.cpp"), "-o", str(exe))
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
