"""The C++ drop-in class (include/torque_gb300/block_sparse.hpp): compiles with
g++ against the library (CPU), and runs the reference's known-answer cases
written against it (GPU)."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "cpp", "block_sparse_kat.cpp")
SRC_DS = os.path.join(ROOT, "tests", "cpp", "dense_sparse_kat.cpp")


def cuda_include():
    for cand in ("/usr/local/cuda/include",):
        if os.path.exists(os.path.join(cand, "cuda_runtime_api.h")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        inc = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
        if os.path.exists(inc):
            return inc
    pytest.skip("CUDA headers not found")


def build_kat(tmp_path, src=SRC):
    from torque_gb300 import build as tq_build
    lib = tq_build.build()
    exe = str(tmp_path / os.path.splitext(os.path.basename(src))[0])
    libdir = os.path.dirname(lib)
    cuda_lib = os.path.join(os.path.dirname(cuda_include()), "lib64")
    # the CUDA runtime too: the move-in case allocates its buffer with cudaMalloc
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"),
           "-I" + cuda_include(), "-o", exe, src, "-L" + libdir, "-ltorque_gb300",
           "-Wl,-rpath," + libdir, "-L" + cuda_lib, "-lcudart", "-Wl,-rpath," + cuda_lib]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_header_compiles(tmp_path):
    build_kat(tmp_path)
    build_kat(tmp_path, SRC_DS)


@pytest.mark.gpu
def test_cpp_known_answers(tq, tmp_path):
    exe = build_kat(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "OK" in r.stdout


@pytest.mark.gpu
def test_cpp_dense_sparse_known_answers(tq, tmp_path):
    exe = build_kat(tmp_path, SRC_DS)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "OK" in r.stdout
