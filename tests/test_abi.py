"""The C-ABI library loads without a GPU and exports every function that
include/fricc_gb300.h declares, with the prototypes the Python binding uses.
Argument checks that fail before any CUDA work are exercised here too."""
import ctypes
import os
import re

import pytest

from conftest import REPO


def _declared():
    src = open(os.path.join(REPO, "include", "fricc_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fricc_[a-z0-9_]+)\s*\(", src)))


def test_header_symbols_exported(gpulib):
    names = _declared()
    assert len(names) >= 14
    for n in names:
        assert hasattr(gpulib, n), n
    from fricc_gb300 import _lib
    bound = {s[0] for s in _lib.SIGNATURES}
    assert bound == set(names), set(names) ^ bound


def test_version_and_error_paths(gpulib):
    assert gpulib.fricc_version() == 100
    from fricc_gb300 import _lib
    # unknown term: rejected before any device work
    d = _lib.i64arr([1, 1, 1, 1])
    st = gpulib.fricc_contract(b"9999", None, d, d, None, None, d, d, None)
    assert st == 2  # FRICC_ERR_TERM
    assert b"CASE NOT IMPLEMENTED" in gpulib.fricc_last_error()
    h = ctypes.c_void_p()
    st = gpulib.fricc_sp_create(None, d, 1, 0, 0, 0.5, None, ctypes.byref(h))
    assert st == 1  # FRICC_ERR_ARG
    with pytest.raises(ValueError):
        _lib.check(st)
