"""ctypes binding of libfricc_gb300.so (the C ABI in include/fricc_gb300.h).

The library is built in-tree (``python -m fricc_gb300.build`` or
``__graft_entry__.build()``).  Loading fails loudly when it is missing: there
is no CPU fallback behind this module.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libfricc_gb300.so")

FRICC_OK = 0
STATUS_NAMES = {1: "FRICC_ERR_ARG", 2: "FRICC_ERR_TERM", 3: "FRICC_ERR_P_GT_ONE", 4: "FRICC_ERR_CUDA",
                5: "FRICC_ERR_TIMEOUT", 6: "FRICC_ERR_INDEX", 7: "FRICC_ERR_UNSUPPORTED", 8: "FRICC_ERR_PIVOTAL"}
COMPRESSION = {"fri": 0, "largest": 1}
SAMPLING = {"systematic": 0, "pivotal": 1}

# (name, restype, argtypes) of every exported symbol
_i64 = ctypes.c_int64
_i64p = ctypes.POINTER(ctypes.c_int64)
_dp = ctypes.c_void_p
_vp = ctypes.c_void_p
_u32p = ctypes.POINTER(ctypes.c_uint32)
_vpp = ctypes.POINTER(ctypes.c_void_p)  # an array of pointers
SIGNATURES = [
    ("fricc_version", ctypes.c_int, []),
    ("fricc_last_error", ctypes.c_char_p, []),
    ("fricc_sp_create", ctypes.c_int, [_dp, _i64p, _i64, ctypes.c_int, ctypes.c_int, ctypes.c_double, _vp,
                                       ctypes.POINTER(_vp)]),
    ("fricc_sp_recompress", ctypes.c_int, [_vp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_double, _vp]),
    ("fricc_sp_create_pivotal", ctypes.c_int, [_dp, _i64p, _i64, _u32p, _vp, ctypes.POINTER(_vp), _i64p]),
    ("fricc_sp_recompress_pivotal", ctypes.c_int, [_vp, _dp, _u32p, _vp, _i64p]),
    ("fricc_sp_status", ctypes.c_int, [_vp]),
    ("fricc_sp_recompress_dev", ctypes.c_int, [_vp, _dp, ctypes.c_int, ctypes.c_int, _dp, _vp]),
    ("fricc_sp_recompress_pair", ctypes.c_int, [_vp, _vp, _dp, ctypes.c_double, ctypes.c_double, _vp]),
    ("fricc_sp_recompress_pair_dev", ctypes.c_int, [_vp, _vp, _dp, _dp, _vp]),
    ("fricc_sp_create_empty", ctypes.c_int, [_i64p, _i64, _vp, ctypes.POINTER(_vp)]),
    ("fricc_sp_destroy", ctypes.c_int, [_vp]),
    ("fricc_sp_info", ctypes.c_int, [_vp, _i64p, _i64p, _i64p]),
    ("fricc_sp_get", ctypes.c_int, [_vp, _i64, _i64p, ctypes.POINTER(ctypes.c_double)]),
    ("fricc_sp_export", ctypes.c_int, [_vp, _vp, _vp, _vp]),
    ("fricc_sp_device_arrays", ctypes.c_int, [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_vp)]),
    ("fricc_contract", ctypes.c_int, [ctypes.c_char_p, _dp, _i64p, _i64p, _vp, _dp, _i64p, _i64p, _vp]),
    ("fricc_contract_batch", ctypes.c_int, [ctypes.c_char_p, _i64, _vpp, _i64p, _i64p, _vpp, _vpp, _i64p, _i64p,
                                            _vp]),
    ("fricc_sp_recompress_batch", ctypes.c_int, [_i64, _vpp, _vpp, ctypes.c_int, ctypes.c_int,
                                                 ctypes.POINTER(ctypes.c_double), _vp]),
    ("fricc_spmm", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                  _dp, _i64, _dp, _vp]),
    ("fricc_spmm_f2", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_double, _dp, _i64, _dp, _vp]),
    ("fricc_split_f2", ctypes.c_int, [_dp, _i64, _i64, _dp, _vp]),
    ("fricc_spmm_f1", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_double, _dp, _i64, _i64, _dp, _vp]),
    ("fricc_spmm_f32", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_double, _dp, _i64, _i64, _dp, _vp]),
    ("fricc_densify_bf16x3", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_double, _vp, _i64, _vp]),
    ("fricc_vvvv_rebuild_split_b", ctypes.c_int, [_vp, _vp, _i64, _i64, _vp, _i64, _vp, _vp]),
    ("fricc_gemm_bf16_tn", ctypes.c_int, [_vp, _i64, _vp, _i64, _i64, _i64, _i64, _dp, _i64, _vp]),
    ("fricc_gemm_bf16_tn_f64", ctypes.c_int, [_vp, _i64, _vp, _i64, _i64, _i64, _i64, _dp, _i64, _vp]),
    ("fricc_split_bf16x3", ctypes.c_int, [_dp, _i64, _i64, _i64, _i64, _vp, _vp, _vp]),
    ("fricc_vvvv_rebuild_bf16x3", ctypes.c_int, [_vp, _vp, _i64, _i64, _dp, _i64, _vp, _vp]),
    ("fricc_split_bf16x3_strided", ctypes.c_int, [_dp, _i64, _i64, _i64, _i64, _i64, _i64, _i64, _vp, _vp, _vp]),
    ("fricc_gemm_bf16_tn_strided", ctypes.c_int, [_vp, _i64, _vp, _i64, _i64, _i64, _i64, _dp, _i64, _i64, _i64,
                                                  _i64, _i64, _i64, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                                  _vp, _vp]),
    ("fricc_gemm_df", ctypes.c_int, [_dp, _dp, _dp, _i64, _i64, _i64, _i64, _i64p, _i64p, _i64p, ctypes.c_double,
                                      ctypes.c_double, _vp]),
    ("fricc_gemm_f64", ctypes.c_int, [_dp, _dp, _dp, _i64, _i64, _i64, _i64, _i64p, _i64p, _i64p, ctypes.c_double,
                                       ctypes.c_double, _vp]),
    ("fricc_combine", ctypes.c_int, [_i64p, ctypes.c_int, _vpp, _i64p, ctypes.c_int, _vpp, _i64p, ctypes.c_int,
                                      _vpp, _i64p, ctypes.POINTER(ctypes.c_double), ctypes.c_int, _vp]),
    ("fricc_zero", ctypes.c_int, [_vp, _i64, _vp]),
    ("fricc_gemm_f64_b2", ctypes.c_int, [_dp, _dp, _dp, _i64, _i64, _i64, _i64, _i64, _i64p, _i64p, _i64p,
                                          ctypes.c_double, ctypes.c_double, _vp]),
    ("fricc_gemm_df_b2", ctypes.c_int, [_dp, _dp, _dp, _i64, _i64, _i64, _i64, _i64, _i64p, _i64p, _i64p,
                                         ctypes.c_double, ctypes.c_double, _vp]),
    ("fricc_combine5", ctypes.c_int, [_i64p, ctypes.c_int, _vpp, _i64p, ctypes.c_int, _vpp, _i64p, ctypes.c_int,
                                       _vpp, _i64p, ctypes.POINTER(ctypes.c_double), ctypes.c_int, _vp]),
    ("fricc_spb_create", ctypes.c_int, [ctypes.c_int, _i64p, _i64, _vp, ctypes.POINTER(_vp)]),
    ("fricc_spb_destroy", ctypes.c_int, [_vp]),
    ("fricc_spb_recompress_pair", ctypes.c_int, [_vp, _dp, _dp, _vp]),
    ("fricc_spb_status", ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int)]),
    ("fricc_spb_export", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp]),
    ("fricc_spb_spmm", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_double, _dp, _i64, _i64, _dp, _i64, _vp]),
    ("fricc_spb_spmm_f2", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_double, _vp, _i64, _i64, _dp, _i64, _vp]),
    ("fricc_symadd_b", ctypes.c_int, [_dp, _dp, _i64, _i64, _i64, _i64p, ctypes.c_double, _vp]),
    ("fricc_spb_densify_bf16x3", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                 ctypes.c_int, ctypes.c_double, _vp, _i64, _vp]),
    ("fricc_gemm_bf16_tn_strided_b", ctypes.c_int, [_vp, _i64, _vp, _i64, _i64, _i64, _i64, _dp, _i64, _i64, _i64,
                                                     _i64, _i64, _i64, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                                     ctypes.c_int, _i64, _i64, _i64, _vp, _vp]),
    ("fricc_energy_update_batch", ctypes.c_int, [ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _i64, _i64, _dp,
                                                 _dp, _dp, _vp]),
    ("fricc_phase_timing_set", ctypes.c_int, [ctypes.c_int]),
    ("fricc_phase_timing_read", ctypes.c_int, [ctypes.POINTER(ctypes.c_double)]),
    ("fricc_contract_flops", ctypes.c_double, [ctypes.c_char_p, _vp]),
    ("fricc_compress", ctypes.c_int, [_dp, _i64, _i64, ctypes.c_int, ctypes.c_double, _dp, _dp, _i64p, _vp]),
    ("fricc_compress_pivotal", ctypes.c_int, [_dp, _i64, _i64, _u32p, _dp, _dp, _i64p, _i64p, _vp]),
    ("fricc_glibc_uniforms", ctypes.c_int, [_u32p, _i64, _dp, _vp]),
    ("fricc_parallel_sample", ctypes.c_int, [_dp, _i64, _i64, ctypes.c_int, _u32p, _dp, _i64p, _vp]),
    ("fricc_seq_cumsum", ctypes.c_int, [_dp, _i64, _dp, _vp]),
    ("fricc_seq_cumsum_noalloc", ctypes.c_int, [_dp, _i64, _dp, _vp]),
    ("fricc_stream_create", ctypes.c_int, [ctypes.POINTER(_vp)]),
    ("fricc_stream_destroy", ctypes.c_int, [_vp]),
    ("fricc_launch_count", ctypes.c_longlong, []),
    ("fricc_alloc_count", ctypes.c_longlong, []),
    ("fricc_tune_set", ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    ("fricc_symadd", ctypes.c_int, [_dp, _dp, _i64, _i64, _i64p, ctypes.c_double, _vp]),
    ("fricc_prof_enable", None, [ctypes.c_int]),
    ("fricc_prof_read", ctypes.c_int, [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong),
                                       ctypes.POINTER(ctypes.c_double)]),
    ("fricc_prof_read_tc", ctypes.c_int, [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong),
                                          ctypes.POINTER(ctypes.c_double)]),
    ("fricc_prof_read_gemm", ctypes.c_int, [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong),
                                            ctypes.POINTER(ctypes.c_double)]),
    ("fricc_energy_update", ctypes.c_int, [_dp, _dp, _dp, _dp, _dp, _dp, _dp, _i64, _i64, _dp, _dp, _dp, _vp]),
    ("fricc_energy_update_lin", ctypes.c_int, [_dp, _dp, _dp, _dp, _dp, _dp, _dp, _i64, _i64, _dp, _dp, _dp, _vp]),
]

_lib = None


class FriccError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def load(path: str = LIB_PATH):
    """Load the shared library (once) and declare every prototype."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(
            f"{path} is missing: build the CUDA library first (python -m fricc_gb300.build); "
            "the GPU path has no CPU fallback")
    L = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(status: int) -> None:
    if status != FRICC_OK:
        msg = load().fricc_last_error()
        msg = msg.decode() if msg else ""
        if status == 1:
            raise ValueError(f"FRICC_ERR_ARG: {msg}")
        if status == 7:
            raise NotImplementedError(f"FRICC_ERR_UNSUPPORTED: {msg}")
        raise FriccError(status, msg)


def i64arr(vals):
    return (ctypes.c_int64 * len(vals))(*[int(v) for v in vals])


def hist_arg(rng):
    """(ctypes uint32[31] or None, writeback) for a draw source: a GlibcRand-like
    object with history()/set_history() lends its history (the device draws
    from it and hands it back); anything else (None, libc's rand) means the
    process's own rand(), as the reference draws."""
    if rng is not None and hasattr(rng, "history") and hasattr(rng, "set_history"):
        h = (ctypes.c_uint32 * 31)(*[int(v) for v in rng.history()])

        def writeback():
            rng.set_history([h[i] for i in range(31)])
        return h, writeback
    return None, (lambda: None)


class OwnStream:
    """A CUDA stream created for one owner (not taken from torch's shared
    stream pool), usable as a torch stream; released with the object."""

    def __init__(self, device):
        import torch
        self._lib = load()
        h = ctypes.c_void_p()
        with torch.cuda.device(device):
            check(self._lib.fricc_stream_create(ctypes.byref(h)))
        self.handle = h
        self.stream = torch.cuda.ExternalStream(h.value, device=device)

    def __del__(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            try:
                self._lib.fricc_stream_destroy(self.handle)
            except Exception:
                pass
            self.handle = None


def cur_stream() -> ctypes.c_void_p:
    """This thread's current CUDA stream on the current device (torch's
    current stream) as a C pointer, read without torch.cuda's Python
    wrappers: an iteration asks for it a few hundred times, and the wrapped
    lookup cost more host time than some of the launches it feeds."""
    import torch
    return ctypes.c_void_p(torch._C._cuda_getCurrentRawStream(torch._C._cuda_getDevice()))
