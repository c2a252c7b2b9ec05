"""The Armadillo API subset the reference's CPU code is compiled against
(oracle/arma_api/armadillo), unit-tested on hand-computed values
(tests/cpp/arma_api_test.cpp): shapes and zeroing of constructors,
column-major access, bounds errors, column/row references, rows/cols/shed/
insert, joins with empty operands, repmat, transposes, reductions, relations,
find, stable sort_index and the matrix product."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "cpp", "arma_api_test.cpp")
SHIM = os.path.join(ROOT, "oracle", "arma_api")


def test_arma_api_subset(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "arma_api_test")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I" + SHIM, "-o", exe, SRC],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok ")
