"""The C ABI library loads and exports every entry point include/*.h declares;
argument checks that return before any device work (CPU only)."""
import ctypes
import glob
import os
import re

import pytest

from conftest import ROOT
from torque_gb300 import _lib
from torque_gb300 import build as tq_build


@pytest.fixture(scope="module")
def lib():
    tq_build.build()
    return _lib.load()


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(tq_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "tq_bs_contract" in names and "tq_bs_create" in names and len(names) >= 20


def test_every_declared_symbol_is_exported(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, "no ctypes signature for " + name


def test_invalid_arguments_return_status(lib):
    out = ctypes.c_void_p()
    dim = (ctypes.c_int64 * 2)(4, 3)
    st = lib.tq_bs_create(_lib.TQ_F64, 2, dim, 0, None, None, None, None, 0, None,
                          ctypes.byref(out))
    assert st == _lib.TQ_ERR_INVALID
    assert b"Source data not allocated" in lib.tq_last_error_string()
    assert lib.tq_bs_contract(None, None, 0, None, None, None, None, ctypes.byref(out)) == \
        _lib.TQ_ERR_INVALID
    assert lib.tq_bs_hard_transpose(None, None, None, None) == _lib.TQ_ERR_INVALID
    assert lib.tq_plan_execute(None, None) == _lib.TQ_ERR_INVALID
    assert lib.tq_bs_destroy(None) == _lib.TQ_OK


def test_adopt_rejects_before_taking_the_buffer(lib):
    """tq_bs_adopt (the move-in constructor) checks its arguments before it
    owns anything: a NULL output or buffer, an unknown type, a rank above 12
    and a box outside the dimension are refused, and the caller keeps the
    buffer (here a host address that must never be freed by the library)."""
    out = ctypes.c_void_p()
    dim = (ctypes.c_int64 * 2)(4, 3)
    b = (ctypes.c_int64 * 2)(0, 0)
    e = (ctypes.c_int64 * 2)(1, 1)
    keep = (ctypes.c_double * 4)()
    buf = ctypes.cast(keep, ctypes.c_void_p)
    assert lib.tq_bs_adopt(_lib.TQ_F64, 2, dim, 1, b, e, None, None, buf, None) == \
        _lib.TQ_ERR_INVALID
    assert lib.tq_bs_adopt(_lib.TQ_F64, 2, dim, 1, b, e, None, None, None,
                           ctypes.byref(out)) == _lib.TQ_ERR_INVALID
    assert b"Source data not allocated" in lib.tq_last_error_string()
    assert lib.tq_bs_adopt(7, 2, dim, 1, b, e, None, None, buf, ctypes.byref(out)) == \
        _lib.TQ_ERR_INVALID
    assert lib.tq_bs_adopt(_lib.TQ_F64, 13, dim, 1, b, e, None, None, buf,
                           ctypes.byref(out)) == _lib.TQ_ERR_UNSUPPORTED
    far = (ctypes.c_int64 * 2)(4, 1)   # leg 0 ends at 4, outside dimension 4
    assert lib.tq_bs_adopt(_lib.TQ_F64, 2, dim, 1, b, far, None, None, buf,
                           ctypes.byref(out)) == _lib.TQ_ERR_INVALID
    assert not out.value
