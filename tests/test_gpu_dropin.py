"""The drop-in boundary, checked against the reference's own driver.

tests/golden/dropin.npz holds every call the unmodified fricc/friccsd.py
(two iterations of its kernel, on the PySCF stand-in) made into the
reference's py_rccsd module: each SparseTensor4d(t2, shape, m, "fri",
"systematic", verbose) with the libc draw it consumed and all its entries,
and each contract_DTSpT(W, T, ouput, term) with W and ouput in the memory
layout the driver passed (transposed views included) and ouput before and
after the call.  Replaying the calls in order through fricc_gb300.py_rccsd
(host numpy arguments, as the driver passes them) must give the same
entries bit for bit and the same outputs to 1e-12 of their scale -- so the
reference's driver, importing this module as fricc.py_rccsd, runs the same
iteration on the GPU."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def _view(data, perm):
    """A C-contiguous copy of data, viewed in the recorded argument's
    index order (so its strides are the recorded argument's)."""
    return np.ascontiguousarray(data).copy().transpose(np.argsort(perm))


def test_replay_reference_driver_calls(gpulib):
    from fricc_gb300 import py_rccsd
    g = golden("dropin.npz")
    tensors = {}
    n_sp = n_ct = 0
    for i in range(int(g["n_calls"])):
        c = lambda key: g[f"c{i}_{key}"]  # noqa: E731
        if str(c("kind")) == "sp":
            x = np.ascontiguousarray(c("x"))
            T = py_rccsd.SparseTensor4d(x, tuple(int(d) for d in c("dims")), int(c("m")), str(c("compression")),
                                        str(c("sampling")), False, rn=float(c("rn")))
            idx, val = T.indices()
            assert np.array_equal(idx, c("idx")), i
            assert np.array_equal(val.view(np.int64), c("val").view(np.int64)), i
            tensors[int(c("k"))] = T
            n_sp += 1
        else:
            W = _view(c("W"), c("wperm"))
            out = _view(c("before"), c("operm"))
            py_rccsd.contract_DTSpT(W, tensors[int(c("sp"))], out, str(c("term")))
            want = np.ascontiguousarray(c("after")).transpose(np.argsort(c("operm")))
            scale = np.abs(want).max() + np.abs(c("before")).max()
            assert np.abs(out - want).max() <= 1e-12 * scale, (i, str(c("term")))
            n_ct += 1
    assert n_sp == 4 and n_ct == 22
