"""Drop-in replacement for fri-cc's ``py_rccsd`` extension module, on the GPU.

Same names, arguments, argument meanings and results as the reference's
pybind11 module (src/py_rccsd.cpp:16-56), so ``fricc/friccsd.py`` can import
it unchanged (``from .py_rccsd import SparseTensor4d, contract_DTSpT``):

* ``SparseTensor4d(tensor_arr, dims, m, compression="fri",
  sampling_method="pivotal", verbose=False)`` -- compresses on the GPU; the
  entries, their order and their values are bit for bit those of the
  reference's single-threaded C++ for the same input and the same libc
  ``rand()`` stream.  ``SparseTensor4d(dims, nnz)`` gives an all-zero tensor.
* ``.get_element(mi) -> ([i, j, a, b], value)`` and ``.print()``.
* ``contract_DTSpT(W, T, ouput, term)`` -- accumulates in place into
  ``ouput`` (the reference's spelling of the keyword), any strides.

Arrays may be numpy (host: copied to the device and, for ``ouput``, back) or
torch CUDA tensors (used in place, on the current torch stream).

Sampling: "systematic" consumes one libc ``rand()``; "pivotal" (the
binding's default) one per element it visits, from this process's ``rand()``
as the reference does, or, with ``rng=GlibcRand(...)``, from that stream
(generated on the device, the object advanced past the draws).  Pivotal
sampling emits S in the reference's order (not sorted).

Differences, all raising instead of terminating the process:
* a bad m, dims, term or compression raises ValueError where the reference
  calls exit(EXIT_FAILURE); a probability above 1 and the pivotal sampler's
  own failures raise FriccError;
* an unknown sampling_method raises ValueError (the reference's check of it
  can never fire, src/fri_utils.cpp:443-455, and its sampled slots then keep
  index 0).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib as L

RAND_MAX = 2147483647
TERMS = ("0101", "2323", "1302", "1202", "1303", "1203", "1323", "0112", "0113", "0313", "0312")

_libc = ctypes.CDLL(None)
_libc.rand.restype = ctypes.c_int


def libc_uniform() -> float:
    """The reference's single draw, rand()/RAND_MAX (src/fri_utils.cpp:47)."""
    return float(_libc.rand()) / float(RAND_MAX)


def parallel_sample(n_sample: int, probs, chunks: int = 1, rng=None) -> np.ndarray:
    """parallel_sample(n_sample, probs) of src/fri_utils.cpp:176-362 (argument
    names of the binding, src/py_rccsd.cpp:22-23) on the GPU: pivotal
    sampling of probs cut into `chunks` chunks (the reference's OpenMP
    threads), each chunk walked by its own warp.  Draws from the process's
    rand() (the reference's stream) or from rng (a GlibcRand), in chunk order.
    Returns the n_sample indices (numpy int64)."""
    lib = L.load()
    qd = _to_device(np.ascontiguousarray(probs, dtype=np.float64) if not isinstance(probs, torch.Tensor) else probs)
    qd = qd.contiguous()
    S = torch.empty(max(int(n_sample), 1), dtype=torch.int64, device=qd.device)
    hist, writeback = L.hist_arg(rng)
    used = ctypes.c_int64(0)
    L.check(lib.fricc_parallel_sample(ctypes.c_void_p(qd.data_ptr()), qd.numel(), int(n_sample), int(chunks), hist,
                                      ctypes.c_void_p(S.data_ptr()), ctypes.byref(used), _stream()))
    writeback()
    return S[:int(n_sample)].cpu().numpy()


def _stream() -> ctypes.c_void_p:
    return L.cur_stream()


def _to_device(a, dtype=torch.float64):
    if isinstance(a, torch.Tensor):
        if not a.is_cuda:
            return a.to("cuda")
        return a
    return torch.from_numpy(np.asarray(a)).to("cuda")


def print_phase_table(sec):
    """The verbose timing table of fri_compression (src/fri_utils.cpp:509-519):
    Sorting, P vector, Sampling, Wrap up and Total seconds, with each one's
    fraction of the total, in the reference's layout."""
    total = sec[4]
    print("Subsection    Fraction of Total    Total Time")
    print("==========    =================    ==========")
    for name, t in zip(("Sorting ", "P vector", "Sampling", "Wrap up ", "Total   "), sec):
        frac = t / total if total > 0 else float("nan")
        print(f"{name}      {frac:6.4f}               {t:6.4f} (s)")


class SparseTensor4d:
    """Device-resident compressed tensor (include/sparse_tensor.hpp:13-100)."""

    def __init__(self, tensor_arr, dims=None, m=None, compression="fri", sampling_method="pivotal",
                 verbose=False, rn=None, rng=None):
        lib = L.load()
        self._h = ctypes.c_void_p()
        if m is None and dims is not None and not isinstance(tensor_arr, (np.ndarray, torch.Tensor)):
            # SparseTensor4d(dims, nnz), src/py_rccsd.cpp:33 (nnz bound as a double)
            d = L.i64arr(tensor_arr)
            L.check(lib.fricc_sp_create_empty(d, int(dims), _stream(), ctypes.byref(self._h)))
            self._dims = tuple(int(x) for x in tensor_arr)
            return
        if isinstance(tensor_arr, np.ndarray):
            if tensor_arr.dtype != np.float64 or not tensor_arr.flags.c_contiguous:
                raise TypeError("tensor_arr must be a C-contiguous float64 array (the binding is noconvert)")
        elif isinstance(tensor_arr, torch.Tensor):
            if tensor_arr.dtype != torch.float64 or not tensor_arr.is_contiguous():
                raise TypeError("tensor_arr must be a contiguous float64 tensor")
        else:
            raise TypeError("tensor_arr must be a numpy array or a torch tensor")
        if compression not in L.COMPRESSION:
            raise ValueError(f"The compression method you chose ({compression}) isn't supported: "
                             "compression must be 'largest' or 'fri'")
        self._dims = tuple(int(x) for x in dims)
        m = int(m)
        x = _to_device(tensor_arr)
        if verbose:
            L.check(lib.fricc_phase_timing_set(1))
        samp = L.SAMPLING.get(sampling_method, -1)
        self.draws_used = 0
        if compression == "fri" and samp < 0:
            raise ValueError(f"sampling_method must be 'pivotal' or 'systematic', got {sampling_method!r}")
        if compression == "fri" and samp == L.SAMPLING["pivotal"]:
            hist, writeback = L.hist_arg(rng)
            used = ctypes.c_int64(0)
            L.check(lib.fricc_sp_create_pivotal(ctypes.c_void_p(x.data_ptr()), L.i64arr(self._dims), m, hist,
                                                _stream(), ctypes.byref(self._h), ctypes.byref(used)))
            writeback()
            self.draws_used = used.value
        else:
            if rn is None:
                rn = (rng() if rng is not None else libc_uniform()) if compression == "fri" else 0.0
            L.check(lib.fricc_sp_create(ctypes.c_void_p(x.data_ptr()), L.i64arr(self._dims), m,
                                        L.COMPRESSION[compression], max(samp, 0), float(rn), _stream(),
                                        ctypes.byref(self._h)))
            L.check(lib.fricc_sp_status(self._h))  # the reference's constructor fails on the spot
        self._keep = x  # the device copy stays alive while the stream may still read it
        if verbose:
            sec = (ctypes.c_double * 5)()
            try:
                L.check(lib.fricc_phase_timing_read(sec))
            finally:
                lib.fricc_phase_timing_set(0)
            print_phase_table(list(sec))

    # -- accessors --------------------------------------------------------
    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def dimension(self, i):
        return self._dims[i]

    def dimensions(self):
        return self._dims

    def size(self):
        m = ctypes.c_int64()
        L.check(L.load().fricc_sp_info(self._h, None, ctypes.byref(m), None))
        return m.value

    def n_largest(self):
        nd = ctypes.c_int64()
        L.check(L.load().fricc_sp_info(self._h, None, None, ctypes.byref(nd)))
        return nd.value

    def get_element(self, mi):
        idx = (ctypes.c_int64 * 4)()
        v = ctypes.c_double()
        L.check(L.load().fricc_sp_get(self._h, int(mi), idx, ctypes.byref(v)))
        return [int(i) for i in idx], float(v.value)

    def export(self):
        """(flat C-order indices, values) of all entries, as numpy arrays."""
        m = self.size()
        flat = np.empty(m, dtype=np.int64)
        vals = np.empty(m, dtype=np.float64)
        L.check(L.load().fricc_sp_export(self._h, ctypes.c_void_p(flat.ctypes.data),
                                         ctypes.c_void_p(vals.ctypes.data), _stream()))
        return flat, vals

    def indices(self):
        flat, vals = self.export()
        return np.stack(np.unravel_index(flat, self._dims), axis=1), vals

    def print(self):
        idx, vals = self.indices()
        print("i   j   k   l        val")
        for r, v in zip(idx, vals):
            print(f"{r[0]}   {r[1]}   {r[2]}   {r[3]}        {v}")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and L._lib is not None:
            L._lib.fricc_sp_destroy(h)
            self._h = ctypes.c_void_p()


def _shape_strides(t: torch.Tensor):
    return L.i64arr(t.shape), L.i64arr(t.stride())


def contract_DTSpT(W, T, ouput, term):
    """``ouput += term(W, T)`` in place (src/sparse_tensor.cpp:349-382)."""
    if term not in TERMS:
        raise ValueError(f"CASE NOT IMPLEMENTED: contraction term {term!r}")
    lib = L.load()
    host_out = None
    if isinstance(ouput, np.ndarray):
        if ouput.dtype != np.float64 or ouput.ndim != 4:
            raise TypeError("ouput must be a float64 4-D array")
        host_out = torch.from_numpy(ouput)
        out_d = host_out.to("cuda")
    else:
        out_d = ouput
    if isinstance(W, np.ndarray):
        if W.dtype != np.float64 or W.ndim != 4:
            raise TypeError("W must be a float64 4-D array")
        W_d = torch.from_numpy(W).to("cuda")
    else:
        W_d = W
    wd, ws = _shape_strides(W_d)
    od, os_ = _shape_strides(out_d)
    L.check(lib.fricc_contract(term.encode(), ctypes.c_void_p(W_d.data_ptr()), wd, ws, T.handle,
                               ctypes.c_void_p(out_d.data_ptr()), od, os_, _stream()))
    if host_out is not None:
        host_out.copy_(out_d)  # blocking device-to-host copy back into the caller's array


def contract_DTSpT_experimental(W, T, ouput, term):
    """The reference's benchmark-only 2323 variants ("taskloop", "atomic",
    src/sparse_tensor.cpp:389-459) compute the 2323 term; so does this."""
    if term not in ("taskloop", "atomic"):
        raise ValueError(f"CASE NOT IMPLEMENTED: {term!r}")
    contract_DTSpT(W, T, ouput, "2323")


def fri_compression(x, n_sample, sampling_method="pivotal", verbose=False, rn=None):
    """(indices, values) of the FRI compression of a flat vector (src/fri_utils.cpp:439-522)."""
    arr = x if isinstance(x, torch.Tensor) else np.ascontiguousarray(x, dtype=np.float64)
    n = int(arr.numel() if isinstance(arr, torch.Tensor) else arr.size)
    t = SparseTensor4d(arr.reshape(-1) if isinstance(arr, np.ndarray) else arr.reshape(-1),
                       (1, 1, 1, n), n_sample, "fri", sampling_method, verbose, rn=rn)
    flat, vals = t.export()
    return flat.tolist(), vals.tolist()
