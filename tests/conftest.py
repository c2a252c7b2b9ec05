import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def load_kat():
    with open(os.path.join(GOLDEN, "kat_block_sparse.json")) as f:
        return json.load(f)


def kat_spec(kat, spec):
    """Resolve a contraction operand spec (a dict, "A", or another case's name)."""
    if isinstance(spec, dict):
        return spec
    for c in kat["contractions"]:
        if c["name"] == spec:
            return c["A"]
    raise KeyError(spec)


def spec_arrays(spec):
    """(dimension, begin [nb, r], end, tables, data) from a KAT operand spec."""
    r = len(spec["dimension"])
    blocks = spec["blocks"]
    b = np.array([x["begin"] for x in blocks], np.int64).reshape(len(blocks), r)
    e = np.array([x["end"] for x in blocks], np.int64).reshape(len(blocks), r)
    has_t = bool(blocks) and all("table" in x for x in blocks)
    t = np.array([x["table"] for x in blocks], np.int64).reshape(len(blocks), r) if has_t else None
    d = np.concatenate([np.asarray(x["data"], np.float64) for x in blocks]) if blocks \
        else np.zeros(0)
    return np.asarray(spec["dimension"], np.int64), b, e, t, d


@pytest.fixture(scope="session")
def kat():
    return load_kat()


def cuda_ok():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def tq():
    """The built library (GPU tests only)."""
    if not cuda_ok():
        pytest.fail("GPU test without a CUDA device: run `pytest -m 'not gpu'` on CPU hosts")
    import torque_gb300
    from torque_gb300 import build as b
    b.build()
    torque_gb300.load()
    return torque_gb300
