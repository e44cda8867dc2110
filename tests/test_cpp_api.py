"""The reference's Rust tests ported to the C++ mirror of its API
(include/scirs_sparse.hpp, tests/cpp/test_reference_api.cpp)."""
import os
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(REPO, "tests", "cpp", "test_reference_api.cpp")
LIBDIR = os.path.join(REPO, "scirs_gb300")


def _compile(out):
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(REPO, "include"), SRC, "-o", out,
           "-L", LIBDIR, "-lscirs_sparse_gpu", f"-Wl,-rpath,{LIBDIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_cpp_mirror_compiles(tmp_path):
    _compile(str(tmp_path / "api_tests"))


@pytest.mark.gpu
def test_cpp_mirror_runs_reference_tests(tmp_path):
    exe = str(tmp_path / "api_tests")
    _compile(exe)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "FAIL" not in r.stdout
