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


def test_python_binding_surface():
    """fricc_gb300.py_rccsd carries the reference binding's names, argument
    names and defaults for the FRI-CCSD path (src/py_rccsd.cpp:22-23,29-30,
    32-54), so keyword calls written for fricc.py_rccsd work unchanged."""
    import inspect

    from fricc_gb300 import py_rccsd as m

    def names(f):
        return list(inspect.signature(f).parameters)

    assert names(m.contract_DTSpT) == ["W", "T", "ouput", "term"]
    assert names(m.contract_DTSpT_experimental) == ["W", "T", "ouput", "term"]
    p = inspect.signature(m.fri_compression).parameters
    assert list(p)[:4] == ["x", "n_sample", "sampling_method", "verbose"]
    assert p["sampling_method"].default == "pivotal" and p["verbose"].default is False
    p = inspect.signature(m.SparseTensor4d.__init__).parameters
    assert list(p)[1:7] == ["tensor_arr", "dims", "m", "compression", "sampling_method", "verbose"]
    assert (p["compression"].default, p["sampling_method"].default, p["verbose"].default) == ("fri", "pivotal", False)
    assert names(m.parallel_sample)[:2] == ["n_sample", "probs"]
    assert callable(m.SparseTensor4d.get_element) and callable(m.SparseTensor4d.print)


def test_binding_argument_checks_before_device_work(gpulib):
    """The binding's own argument errors (src/py_rccsd.cpp:34-39 noconvert,
    include/sparse_tensor.hpp:70-76 unknown compression,
    src/sparse_tensor.cpp:378-381 unknown term) raise before any device work."""
    import numpy as np

    from fricc_gb300 import py_rccsd as m
    a = np.zeros((2, 2, 3, 3))
    with pytest.raises(TypeError):
        m.SparseTensor4d(a.astype(np.float32), a.shape, 4, "fri", "systematic")
    with pytest.raises(TypeError):
        m.SparseTensor4d(np.asfortranarray(a), a.shape, 4, "fri", "systematic")
    with pytest.raises(TypeError):
        m.SparseTensor4d(a.tolist(), a.shape, 4, "fri", "systematic")
    with pytest.raises(ValueError, match="compression"):
        m.SparseTensor4d(a, a.shape, 4, "random")
    with pytest.raises(ValueError, match="CASE NOT IMPLEMENTED"):
        m.contract_DTSpT(a, None, a.copy(), "2332")
    with pytest.raises(ValueError, match="CASE NOT IMPLEMENTED"):
        m.contract_DTSpT_experimental(a, None, a.copy(), "2323")


@pytest.mark.parametrize("compiler,ext", [("gcc", "c"), ("g++", "cpp")])
def test_header_compiles_and_links(gpulib, tmp_path, compiler, ext):
    """A C and a C++ program that include include/fricc_gb300.h, take the
    address of every function it declares and link against the built
    library (the integration a C or C++ host makes) compile, link and run
    fricc_version() without a GPU."""
    import shutil
    import subprocess

    if shutil.which(compiler) is None:
        pytest.skip(f"{compiler} not found")
    names = _declared()
    src = tmp_path / f"probe.{ext}"
    src.write_text(
        '#include "fricc_gb300.h"\n#include <stdio.h>\n'
        "typedef void (*fp)(void);\n"
        "int main(void) {\n  volatile fp f[] = {\n"
        + "".join(f"    (fp){n},\n" for n in names)
        + "  };\n  (void)f;\n  printf(\"%d\\n\", fricc_version());\n  return 0;\n}\n")
    libdir = os.path.join(REPO, "fricc_gb300", "_lib")
    exe = tmp_path / "probe"
    r = subprocess.run([compiler, "-Wall", "-Werror", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe),
                        "-L", libdir, "-lfricc_gb300", f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip() == "100", (r.stdout, r.stderr)


def test_missing_library_fails_loudly(tmp_path, monkeypatch):
    """Without the built library the GPU path raises at load time; nothing
    falls back to a CPU implementation."""
    from fricc_gb300 import _lib
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(ImportError, match="no CPU fallback"):
        _lib.load(str(tmp_path / "libfricc_gb300.so"))


def test_batch_entry_points_check_arguments(gpulib):
    """fricc_contract_batch / fricc_sp_recompress_batch: bad counts and null
    arrays are rejected, count 0 does nothing, and an item's own error (here
    raised before any device work) comes back with its index in front."""
    import ctypes

    from fricc_gb300 import _lib
    d = _lib.i64arr([1] * 8)
    nulls = (ctypes.c_void_p * 2)()
    assert gpulib.fricc_contract_batch(b"2323", -1, nulls, d, d, nulls, nulls, d, d, None) == 1
    assert gpulib.fricc_contract_batch(b"2323", 2, None, d, d, nulls, nulls, d, d, None) == 1
    assert gpulib.fricc_contract_batch(b"2323", 0, None, None, None, None, None, None, None, None) == 0
    assert gpulib.fricc_contract_batch(b"9999", 2, nulls, d, d, nulls, nulls, d, d, None) == 2
    assert gpulib.fricc_last_error().startswith(b"contract_batch item 0: CASE NOT IMPLEMENTED")
    rn = (ctypes.c_double * 2)(0.5, 0.5)
    assert gpulib.fricc_sp_recompress_batch(-1, nulls, nulls, 0, 0, rn, None) == 1
    assert gpulib.fricc_sp_recompress_batch(2, nulls, nulls, 0, 0, None, None) == 1
    assert gpulib.fricc_sp_recompress_batch(0, None, None, 0, 0, None, None) == 0
    assert gpulib.fricc_sp_recompress_batch(2, nulls, nulls, 0, 0, rn, None) == 1
    assert gpulib.fricc_last_error() == b"sp_recompress_batch item 0: sp_recompress: null argument"
