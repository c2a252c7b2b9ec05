"""The reference's own test sources, unchanged.

CPU suites (test/block_sparse_tensor_test.cpp, dense_tensor_test.cpp,
sparse_tensor_test.cpp): built from the reference's sources (src/tensor/*.cpp
and the headers) against the project's Armadillo API subset, with `assert`
enabled as the reference's default build has it, and run: every assertion
passes.  This checks the API subset that the oracle build of the reference
(oracle/build_ref.py) relies on.

GPU suites: they compile and link, unchanged, against the drop-in headers.

test/gpu/block_sparse_test.cu, dense_test.cu, cpu_gpu_comparison.cu,
peps_test.cu, dense_peps_test.cu and the two benchmarks of the reference include "gpu/block_sparse.cuh", "gpu/dense.cuh" and "gpu/sparse.cuh";
tests/ref_suite/ maps those names to include/torque_gb300/block_sparse.hpp,
dense.hpp and sparse.hpp (plus cuBLAS's declarations and the reference's CPU
tensors, as the reference headers bring them in; cpu_gpu_comparison.cu checks
the GPU classes against the reference's CPU classes, linked from its
sources), Armadillo is the project's API subset (oracle/arma_api) and Catch2
is the copy the reference vendors.  The programs are linked against
libtorque_gb300.so and cuBLAS (for the handle the tests create) but not run:
the reference's sources exist only where it is checked out, which has no GPU;
the same known answers run on the GPU through tests/test_gpu_kat.py and
tests/test_cpp_api.py.  Skipped where the reference's sources are absent."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT
from oracle import build_ref

REF = build_ref.reference_root()
SUITE = os.path.join(ROOT, "tests", "ref_suite")

pytestmark = pytest.mark.skipif(REF is None or shutil.which("g++") is None,
                                reason="needs the reference's sources and g++")


def cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(nvcc))


@pytest.fixture(scope="module")
def catch_main(tmp_path_factory):
    obj = str(tmp_path_factory.mktemp("catch") / "catch_main.o")
    r = subprocess.run(["g++", "-std=c++17", "-O0", "-c",
                        "-I" + os.path.join(REF, "external", "catch2"),
                        os.path.join(SUITE, "catch_main.cpp"), "-o", obj],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return obj


@pytest.mark.parametrize("name", ["block_sparse_test", "dense_test", "cpu_gpu_comparison",
                                  "peps_test", "dense_peps_test", "block_sparse_benchmark",
                                  "large_tensor_benchmark"])
def test_reference_gpu_test_builds_against_dropin(tmp_path, catch_main, name):
    from torque_gb300 import build as tq_build
    lib = tq_build.build()
    libdir = os.path.dirname(lib)
    cuda = cuda_home()
    exe = str(tmp_path / name)
    cmd = ["g++", "-std=c++17", "-O0", "-x", "c++",
           "-I" + SUITE, "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "oracle", "arma_api"), "-I" + os.path.join(REF, "src"),
           "-I" + os.path.join(REF, "external", "catch2"), "-I" + os.path.join(cuda, "include"),
           os.path.join(REF, "test", "gpu", name + ".cu"), "-x", "none"] + \
        [os.path.join(REF, "src", "tensor", f) for f in ("block_sparse.cpp", "sparse.cpp",
                                                         "dense.cpp")] + \
        ["-w", catch_main, "-L" + libdir, "-ltorque_gb300", "-Wl,-rpath," + libdir,
         "-L" + os.path.join(cuda, "lib64"), "-lcublas", "-lcudart", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    assert os.path.getsize(exe) > 0


@pytest.mark.parametrize("name", ["block_sparse_tensor_test", "dense_tensor_test",
                                  "sparse_tensor_test"])
def test_reference_cpu_suite_passes(tmp_path, catch_main, name):
    src = os.path.join(REF, "src")
    exe = str(tmp_path / name)
    cmd = ["g++", "-std=c++17", "-O1", "-w", "-I" + os.path.join(ROOT, "oracle", "arma_api"),
           "-I" + src, "-I" + os.path.join(src, "tensor"),
           "-I" + os.path.join(REF, "external", "catch2"),
           os.path.join(REF, "test", name + ".cpp")] + \
        [os.path.join(src, "tensor", f) for f in ("block_sparse.cpp", "sparse.cpp", "dense.cpp")] + \
        [catch_main, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout[-4000:]
    assert "All tests passed" in out.stdout
