"""Python face of the C oracle (oracle/fri_oracle.c).

TEST INFRASTRUCTURE ONLY: the tests, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` use this module to check the CUDA path or to
time the reference algorithm on the host.  The product never imports it.

It mirrors the reference's pybind11 module ``py_rccsd`` (src/py_rccsd.cpp:16-56):
``SparseTensor4d(tensor_arr, dims, m, compression, sampling_method, verbose)``,
``.get_element(mi)``, ``contract_DTSpT(W, T, ouput, term)``, plus
``fri_compression``.  The one uniform draw that systematic sampling makes
(src/fri_utils.cpp:47) comes from libc ``rand()`` through ctypes, i.e. from the
same process-global stream the reference module would use, unless the caller
passes ``rn`` explicitly.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libfri_oracle.so")
_lib = None

RAND_MAX = 2147483647  # glibc
TERMS = ("0101", "2323", "1302", "1202", "1303", "1203", "1323", "0112", "0113", "0313", "0312")

_i64p = ctypes.POINTER(ctypes.c_int64)
_f64p = ctypes.POINTER(ctypes.c_double)


def build(quiet: bool = True) -> str:
    """Compile oracle/fri_oracle.c with oracle/Makefile (gcc, no GPU)."""
    cmd = ["make", "-C", _HERE, "-s"]
    subprocess.run(cmd, check=True, capture_output=quiet)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH) or (
            os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "fri_oracle.c"))
        ):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        L.fo_one_norm.restype = ctypes.c_double
        L.fo_one_norm.argtypes = [_f64p, ctypes.c_int64]
        L.fo_argsort.argtypes = [_f64p, ctypes.c_int64, ctypes.c_int64, _i64p]
        L.fo_fri_compression.argtypes = [_f64p, ctypes.c_int64, ctypes.c_int64, ctypes.c_double,
                                         _i64p, _f64p, _i64p]
        L.fo_largest.argtypes = [_f64p, ctypes.c_int64, ctypes.c_int64, _i64p, _f64p]
        L.fo_fri_compression_pivotal.argtypes = [_f64p, ctypes.c_int64, ctypes.c_int64, _f64p, ctypes.c_int64,
                                                 _i64p, _f64p, _i64p, _i64p]
        L.fo_parallel_sample.argtypes = [ctypes.c_int64, _f64p, ctypes.c_int64, ctypes.c_int, _f64p,
                                         ctypes.c_int64, _i64p, _i64p]
        L.fo_unpack.argtypes = [_i64p, ctypes.c_int64, _i64p, _i64p]
        L.fo_term_id.argtypes = [ctypes.c_char_p]
        L.fo_outer_size.restype = ctypes.c_int64
        L.fo_outer_size.argtypes = [ctypes.c_int, _i64p, _i64p]
        L.fo_contract.argtypes = [ctypes.c_int, _f64p, _i64p, _i64p, _i64p, _f64p, ctypes.c_int64,
                                  _i64p, _f64p, _i64p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64]
        L.fo_get_d_largest.restype = ctypes.c_int64
        L.fo_get_d_largest.argtypes = [_f64p, ctypes.c_int64, ctypes.c_int64, _i64p, _f64p]
        L.fo_max_threads.restype = ctypes.c_int
        L.fo_set_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t)


def libc_rand_uniform() -> float:
    """rn = (double)rand() / RAND_MAX from the process-global libc stream."""
    libc = ctypes.CDLL(None)
    return float(libc.rand()) / float(RAND_MAX)


def libc_srand(seed: int) -> None:
    ctypes.CDLL(None).srand(ctypes.c_uint(seed))


def set_threads(n: int) -> None:
    lib().fo_set_threads(int(n))


def one_norm(x: np.ndarray) -> float:
    x = np.ascontiguousarray(x, dtype=np.float64).ravel()
    return lib().fo_one_norm(_p(x, _f64p), x.size)


def argsort(x: np.ndarray, m: int) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64).ravel()
    out = np.empty(m, dtype=np.int64)
    st = lib().fo_argsort(_p(x, _f64p), x.size, m, _p(out, _i64p))
    if st:
        raise ValueError("argsort: bad arguments")
    return out


def get_d_largest(x: np.ndarray, m: int):
    x = np.ascontiguousarray(x, dtype=np.float64).ravel()
    srt = argsort(x, m)
    R = ctypes.c_double(0.0)
    nd = lib().fo_get_d_largest(_p(x, _f64p), x.size, m, _p(srt, _i64p), ctypes.byref(R))
    return srt[:nd].copy(), R.value


def fri_compression(x: np.ndarray, m: int, rn: float | None = None):
    """Systematic FRI compression; returns (flat_idx[m], vals[m], n_largest)."""
    x = np.ascontiguousarray(x, dtype=np.float64).ravel()
    if rn is None:
        rn = libc_rand_uniform()
    idx = np.empty(m, dtype=np.int64)
    val = np.empty(m, dtype=np.float64)
    nd = ctypes.c_int64(0)
    st = lib().fo_fri_compression(_p(x, _f64p), x.size, m, rn, _p(idx, _i64p), _p(val, _f64p),
                                  ctypes.byref(nd))
    if st == 3:
        raise RuntimeError("ERROR MAKING PROBABILITY VECTOR (p > 1)")
    if st:
        raise ValueError(f"fri_compression: status {st}")
    return idx, val, nd.value


def fri_compression_pivotal(x: np.ndarray, m: int, draws=None):
    """Pivotal FRI compression; returns (flat_idx[m], vals[m], n_largest, draws_used).

    draws: the uniforms rand()/RAND_MAX in order (an array); None draws from
    libc rand() itself, like the reference."""
    x = np.ascontiguousarray(x, dtype=np.float64).ravel()
    idx = np.empty(m, dtype=np.int64)
    val = np.empty(m, dtype=np.float64)
    nd, used = ctypes.c_int64(0), ctypes.c_int64(0)
    if draws is None:
        dp, na = None, 0
    else:
        draws = np.ascontiguousarray(draws, dtype=np.float64)
        dp, na = _p(draws, _f64p), draws.size
    st = lib().fo_fri_compression_pivotal(_p(x, _f64p), x.size, m, dp, na, _p(idx, _i64p), _p(val, _f64p),
                                          ctypes.byref(nd), ctypes.byref(used))
    if st == 3:
        raise RuntimeError("ERROR MAKING PROBABILITY VECTOR (p > 1)")
    if st == 7:
        raise RuntimeError("ERROR IN PIVOTAL SAMPLING")
    if st:
        raise ValueError(f"fri_compression_pivotal: status {st}")
    return idx, val, nd.value, used.value


def parallel_sample(n_sample: int, q: np.ndarray, chunks: int, draws):
    """parallel_sample with `chunks` chunks and the given draws (in chunk
    order); returns (S[n_sample], draws_used)."""
    q = np.ascontiguousarray(q, dtype=np.float64).ravel()
    draws = np.ascontiguousarray(draws, dtype=np.float64)
    S = np.zeros(max(n_sample, 1), dtype=np.int64)
    used = ctypes.c_int64(0)
    st = lib().fo_parallel_sample(n_sample, _p(q, _f64p), q.size, chunks, _p(draws, _f64p), draws.size,
                                  _p(S, _i64p), ctypes.byref(used))
    if st == 7:
        raise RuntimeError("ERROR IN PIVOTAL SAMPLING")
    if st:
        raise ValueError(f"parallel_sample: status {st}")
    return S[:n_sample], used.value


def largest(x: np.ndarray, m: int):
    x = np.ascontiguousarray(x, dtype=np.float64).ravel()
    idx = np.empty(m, dtype=np.int64)
    val = np.empty(m, dtype=np.float64)
    st = lib().fo_largest(_p(x, _f64p), x.size, m, _p(idx, _i64p), _p(val, _f64p))
    if st:
        raise ValueError(f"largest: status {st}")
    return idx, val


def unpack(flat: np.ndarray, dims) -> np.ndarray:
    flat = np.ascontiguousarray(flat, dtype=np.int64)
    d = np.asarray(dims, dtype=np.int64)
    out = np.empty((flat.size, 4), dtype=np.int64)
    st = lib().fo_unpack(_p(flat, _i64p), flat.size, _p(d, _i64p), _p(out, _i64p))
    if st:
        raise IndexError("Indices are out of range for given tensor")
    return out


class SparseTensor4d:
    """Oracle mirror of the reference's SparseTensor4d (include/sparse_tensor.hpp:13-100)."""

    def __init__(self, tensor_arr, dims, m=None, compression="fri", sampling_method="pivotal",
                 verbose=False, rn=None, draws=None):
        if m is None:  # SparseTensor4d(dims, nnz): an empty tensor (src/py_rccsd.cpp:33)
            self.dims = tuple(int(d) for d in tensor_arr)
            nnz = int(dims)
            self.idx4 = np.zeros((nnz, 4), dtype=np.int64)
            self.vals = np.zeros(nnz)
            self.flat = np.zeros(nnz, dtype=np.int64)
            self.n_largest = 0
            return
        if not (isinstance(tensor_arr, np.ndarray) and tensor_arr.dtype == np.float64
                and tensor_arr.flags.c_contiguous):
            raise TypeError("tensor_arr must be a C-contiguous float64 numpy array")
        self.dims = tuple(int(d) for d in dims)
        m = int(m)
        if compression == "largest":
            self.flat, self.vals = largest(tensor_arr, m)
            self.n_largest = m
        elif compression == "fri":
            if sampling_method == "pivotal":
                self.flat, self.vals, self.n_largest, self.draws_used = fri_compression_pivotal(tensor_arr, m, draws)
            elif sampling_method == "systematic":
                self.flat, self.vals, self.n_largest = fri_compression(tensor_arr, m, rn)
            else:
                raise ValueError(f"sampling_method {sampling_method!r}")
        else:
            raise ValueError(f"The compression method you chose ({compression}) isn't supported")
        self.idx4 = unpack(self.flat, self.dims)

    def get_element(self, mi):
        return [int(v) for v in self.idx4[mi]], float(self.vals[mi])

    def dimension(self, i):
        return self.dims[i]

    def size(self):
        return self.vals.size


def _strides(a: np.ndarray) -> np.ndarray:
    return np.asarray([s // 8 for s in a.strides], dtype=np.int64)


def contract_DTSpT(W, T, ouput, term, outer_range=None):
    """Accumulate the sparse x dense term into ``ouput`` in place (src/sparse_tensor.cpp:349-382).

    W and ouput may carry any (element-aligned, non-negative) strides.
    ``outer_range=(begin, end)`` or ``(begin, end, step)`` restricts the
    outer-pair loop to begin, begin + step, ... < end (timing samples).
    """
    if term not in TERMS:
        raise ValueError(f"CASE NOT IMPLEMENTED: {term}")
    for a in (W, ouput):
        if a.dtype != np.float64 or a.ndim != 4:
            raise TypeError("W and ouput must be float64 4-D arrays")
    L = lib()
    tid = L.fo_term_id(term.encode())
    wd = np.asarray(W.shape, dtype=np.int64)
    ws = _strides(W)
    td = np.asarray(T.dims, dtype=np.int64)
    os_ = _strides(ouput)
    idx4 = np.ascontiguousarray(T.idx4, dtype=np.int64)
    vals = np.ascontiguousarray(T.vals, dtype=np.float64)
    b, e, step = (0, -1, 1) if outer_range is None else (tuple(outer_range) + (1,))[:3]
    # ctypes pointers at the array base honour negative-free strides
    st = L.fo_contract(tid, ctypes.cast(W.ctypes.data, _f64p), _p(wd, _i64p), _p(ws, _i64p),
                       _p(idx4, _i64p), _p(vals, _f64p), vals.size, _p(td, _i64p),
                       ctypes.cast(ouput.ctypes.data, _f64p), _p(os_, _i64p), b, e, step)
    if st:
        raise ValueError(f"contract_DTSpT: status {st}")


def outer_size(term: str, tdims, wdims) -> int:
    L = lib()
    td = np.asarray(tdims, dtype=np.int64)
    wd = np.asarray(wdims, dtype=np.int64)
    return int(L.fo_outer_size(L.fo_term_id(term.encode()), _p(td, _i64p), _p(wd, _i64p)))
