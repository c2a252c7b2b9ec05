"""Recipe: compile the reference's own CPU block-sparse code into oracle/_ref/.

TEST INFRASTRUCTURE ONLY.  The reference (Walter-Feng/Torque) keeps its CPU
tensor in header templates (src/tensor/block_sparse.h, dense.h,
src/util/space.h) plus one source file (src/tensor/block_sparse.cpp, the
block matcher).  They need Armadillo, which is not installed; they compile
here, unmodified, against the project's Armadillo API subset
(oracle/arma_api/armadillo).  ``ref_driver.cpp`` puts plain C entry points
over ``BlockSparseTensor<double>``; ``ref.py`` loads them.

Two libraries are built, both with g++ -O2 -DNDEBUG (the reference's CMake
sets no optimisation level of its own; NDEBUG keeps its ``assert`` on a
sorted stride table, which its full-contraction path feeds a dimension
vector, from aborting the test process):

* ``libtorque_ref_asis.so``: the headers exactly as they are;
* ``libtorque_ref_fixed.so``: the same, with the CPU contract's two stride
  lookups corrected (``index_tables.col(j_block)`` -> the pair's own blocks,
  src/tensor/block_sparse.h:531,538).  The corrected header text is fed to
  the compiler on standard input; no copy of it is written anywhere.

The reference's sources exist only where the reference is checked out; on
any other machine ``build()`` returns None and the tests that need these
libraries skip.  Outputs go to oracle/_ref/ only (kept out of version
control).
"""
from __future__ import annotations

import os
import subprocess
import sys

_HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(_HERE, "_ref")
SHIM = os.path.join(_HERE, "arma_api")
DRIVER = os.path.join(_HERE, "ref_driver.cpp")
DEFAULT_ROOT = "/root/reference"

LIBS = {"asis": "libtorque_ref_asis.so", "fixed": "libtorque_ref_fixed.so"}

# The two stride lookups of the CPU contract (block_sparse.h:531,538) read the
# index table of the j_block-th partner instead of the pair's own blocks.
STRIDE_FIXES = (
    ("this->index_tables.col(j_block)", "this->index_tables.col(i)"),
    ("tensor.index_tables.col(j_block)", "tensor.index_tables.col(B_block_index)"),
)

FLAGS = ["-std=c++17", "-O2", "-DNDEBUG", "-fPIC", "-shared", "-Wl,-Bsymbolic", "-w"]


def reference_root() -> str | None:
    root = os.environ.get("TORQUE_REFERENCE_ROOT", DEFAULT_ROOT)
    return root if os.path.isfile(os.path.join(root, "src", "tensor", "block_sparse.h")) else None


def _inputs(root: str) -> list[str]:
    src = os.path.join(root, "src")
    return [os.path.join(src, "tensor", "block_sparse.h"),
            os.path.join(src, "tensor", "block_sparse.cpp"),
            os.path.join(src, "tensor", "dense.h"),
            os.path.join(src, "util", "space.h"),
            os.path.join(src, "error.h"),
            os.path.join(SHIM, "armadillo"), DRIVER, os.path.abspath(__file__)]


def _stale(target: str, inputs: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(p) > t for p in inputs)


def fixed_header_text(root: str) -> str:
    with open(os.path.join(root, "src", "tensor", "block_sparse.h")) as f:
        text = f.read()
    for old, new in STRIDE_FIXES:
        if text.count(old) != 1:
            raise RuntimeError("expected exactly one %r in block_sparse.h" % old)
        text = text.replace(old, new)
    return text


def build(force: bool = False) -> dict | None:
    """Compile both libraries when the reference's sources are present and the
    outputs are out of date.  Returns {variant: path} or None."""
    root = reference_root()
    if root is None:
        return None
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(root, "src")
    inc = ["-I", SHIM, "-I", src, "-I", os.path.join(src, "tensor")]
    matcher = os.path.join(src, "tensor", "block_sparse.cpp")
    ins = _inputs(root)
    paths = {v: os.path.join(OUT, name) for v, name in LIBS.items()}
    jobs = []
    if force or _stale(paths["asis"], ins):
        cmd = ["g++"] + FLAGS + inc + [DRIVER, matcher, "-o", paths["asis"]]
        jobs.append((subprocess.Popen(cmd), None, cmd))
    if force or _stale(paths["fixed"], ins):
        with open(DRIVER) as f:
            tu = fixed_header_text(root) + "\n" + f.read()
        cmd = ["g++"] + FLAGS + inc + ["-x", "c++", "-", "-x", "none", matcher,
                                       "-o", paths["fixed"]]
        p = subprocess.Popen(cmd, stdin=subprocess.PIPE, text=True)
        jobs.append((p, tu, cmd))
    for p, text, cmd in jobs:
        p.communicate(text)
        if p.returncode != 0:
            raise subprocess.CalledProcessError(p.returncode, cmd)
    return paths


if __name__ == "__main__":  # pragma: no cover
    print(build(force="--force" in sys.argv))
