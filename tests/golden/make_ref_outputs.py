"""Write ref_outputs.npz: the outputs of the reference's own CPU
BlockSparseTensor<double> on the cases of ref_cases.py.

Needs the reference's sources: oracle/build_ref.py compiles them (against
the project's Armadillo API subset) into oracle/_ref/, in the variant as it
is ("asis") and with the CPU contract's stride lookups corrected ("fixed").
Run from the repository root:

    python tests/golden/make_ref_outputs.py

For every contraction case and both variants the file holds the output block
list (begin/end [n_blocks, rank], offsets) and either all values (results up
to 4,096 elements) or the per-block digest of ref_cases.value_digest; a
scalar result is stored as such, a case where the reference throws stores
its message, and where the as-is strides would read past a tensor's values
(the oracle's mode 2 detects it) the as-is build is not run and the case is
marked "undefined".  Transposition, query and modify cases store their full
results (for modify: the reads in order and the tensor afterwards).  Keys
are "<case>__<variant>__<field>" (variant "f32": the stride-fixed build's float
instantiation); "<case>__input" is the sha256 of the inputs.
"""
from __future__ import annotations

import os
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(os.path.dirname(_HERE))
for p in (_ROOT, _HERE):
    if p not in sys.path:
        sys.path.insert(0, p)

import ref_cases as rc  # noqa: E402
from oracle import build_ref, ref  # noqa: E402
from oracle import oracle as orc  # noqa: E402

FULL_LIMIT = 4096


def main() -> None:
    if build_ref.build() is None:
        raise SystemExit("the reference's sources are not here; nothing to generate")
    z = {}
    for name, make in rc.CONTRACTIONS.items():
        A, B, pairs = make()
        z[name + "__input"] = np.array(rc.input_digest(A, B))
        z[name + "__pairs"] = pairs
        for v in ("fixed", "asis"):
            key = "%s__%s__" % (name, v)
            if v == "asis":
                try:
                    orc.contract(A, B, pairs, mode=2)
                except orc.UndefinedRead:
                    # the as-is strides would read past the values: undefined
                    z[key + "undefined"] = np.array(True)
                    continue
                except IndexError:
                    pass
            try:
                out = ref.contract(A, B, pairs, variant=v)
            except ref.RefError as e:
                z[key + "error"] = np.array(str(e))
                continue
            if isinstance(out, float):
                z[key + "scalar"] = np.array(out)
                continue
            begin, end, offsets, data = out
            z[key + "begin"], z[key + "end"], z[key + "offsets"] = begin, end, offsets
            if data.size <= FULL_LIMIT:
                z[key + "values"] = data
            else:
                z[key + "digest"] = rc.value_digest(offsets, rc.block_sizes(begin, end), data)
    for name in rc.FLOAT_CASES:
        A, B, pairs = rc.CONTRACTIONS[name]()
        begin, end, offsets, data = ref.contract(A, B, pairs, variant="fixed", dtype=np.float32)
        key = "%s__f32__" % name
        z[key + "begin"], z[key + "end"], z[key + "offsets"] = begin, end, offsets
        if data.size <= FULL_LIMIT:
            z[key + "values"] = data
        else:
            z[key + "digest"] = rc.value_digest(offsets, rc.block_sizes(begin, end),
                                                data.astype(np.float64))
    for tname, T in rc.transpose_cases().items():
        z[tname + "__input"] = np.array(rc.input_digest(T))
        for k, perm in enumerate(rc.TRANSPOSE_PERMS):
            R = ref.hard_transpose(T, perm)
            key = "%s__%d__" % (tname, k)
            z[key + "perm"] = np.asarray(perm, np.int64)
            z[key + "begin"], z[key + "end"] = R.begin, R.end
            z[key + "tables"], z[key + "offsets"], z[key + "values"] = \
                R.strides, R.offsets, R.data
    Q, points = rc.query_r3()
    z["query_r3__input"] = np.array(rc.input_digest(Q))
    z["query_r3__points"] = points
    z["query_r3__values"] = np.array([ref.query(Q, p) for p in points])
    M, ops = rc.modify_r3()
    z["modify_r3__input"] = np.array(rc.input_digest(M))
    R = ref.RefTensor.from_host(M)
    reads = []
    for kind, idx, value in ops:
        if kind == "modify":
            R.modify(idx, value)
        else:
            reads.append(R.query(idx))
    H = R.host()
    z["modify_r3__reads"] = np.asarray(reads, np.float64)
    z["modify_r3__begin"], z["modify_r3__end"] = H.begin, H.end
    z["modify_r3__tables"], z["modify_r3__offsets"], z["modify_r3__values"] = \
        H.strides, H.offsets, H.data
    np.savez_compressed(rc.FIXTURE, **z)
    print("wrote %s (%d arrays, %d bytes)" % (rc.FIXTURE, len(z), os.path.getsize(rc.FIXTURE)))


if __name__ == "__main__":
    main()
