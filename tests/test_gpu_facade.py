"""The C++ drop-in facade (include/ikd_Tree_gb300.h): compiles against the
header as reference user code would, links libikdg, and passes its own
brute-force checks on the GPU (tests/cpp/facade_test.cpp)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _compile(tmp_path):
    lib_dir = os.path.join(ROOT, "ikd-tree_gb300")
    exe = str(tmp_path / "facade_test")
    cmd = ["g++", "-std=c++14", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "facade_test.cpp"), "-o", exe,
           "-L", lib_dir, "-likdg", f"-Wl,-rpath,{lib_dir}", "-L/usr/local/cuda/lib64", "-lcudart"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_facade_compiles(tmp_path):
    # No GPU needed to build against the header.
    assert os.path.exists(_compile(tmp_path))


@pytest.mark.gpu
def test_facade_runs_on_gpu(tmp_path):
    exe = _compile(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "facade ok" in r.stdout
