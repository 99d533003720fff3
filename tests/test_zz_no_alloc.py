"""fricc_seq_cumsum_noalloc, the entry point for callers that cannot
allocate device memory (its scratch is a fixed array inside the library):
called through the C ABI, it must give exactly what the allocating
fricc_seq_cumsum gives, on two calls in a row (the second sees the first
call's leftovers in the shared scratch), and reject sizes above its limit.

This file is collected last on purpose, so a run that stops at the first
failure has already run every other test."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

MAX_N = 1 << 26


def _call(lib, name, x, out):
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    return getattr(lib, name)(ctypes.c_void_p(x.data_ptr()), x.numel(), ctypes.c_void_p(out.data_ptr()), st)


def test_noalloc_matches_allocating_entry_point(gpulib):
    from fricc_gb300 import _lib
    rng = np.random.default_rng(11)
    inputs = [
        np.abs(rng.standard_normal(3_000_001)) * np.exp(4 * rng.standard_normal(3_000_001)),
        np.concatenate([np.zeros(1000), rng.random(250_000)]),   # shorter: old scratch stays behind it
    ]
    for x_h in inputs:
        x = torch.from_numpy(x_h).cuda()
        ref = torch.empty_like(x)
        got = torch.full_like(x, np.nan)
        _lib.check(_call(gpulib, "fricc_seq_cumsum", x, ref))
        _lib.check(_call(gpulib, "fricc_seq_cumsum_noalloc", x, got))
        torch.cuda.synchronize()
        r, g = ref.cpu().numpy(), got.cpu().numpy()
        assert np.array_equal(r.view(np.int64), g.view(np.int64))  # both are exact: bit for bit
        assert np.array_equal(g.view(np.int64), np.add.accumulate(x_h).view(np.int64))


def test_noalloc_at_the_size_limit_allocates_nothing(gpulib):
    """n = 2^26, where the chunk scratch is used to its last entry: still bit
    for bit the allocating entry point's result, and the library's
    allocation counter does not move during the call (the allocating entry
    point, called for contrast, does allocate)."""
    from fricc_gb300 import _lib
    rng = np.random.default_rng(12)
    x_h = rng.random(MAX_N)
    x = torch.from_numpy(x_h).cuda()
    ref = torch.empty_like(x)
    got = torch.empty_like(x)
    torch.cuda.synchronize()
    before = gpulib.fricc_alloc_count()
    _lib.check(_call(gpulib, "fricc_seq_cumsum_noalloc", x, got))
    torch.cuda.synchronize()
    assert gpulib.fricc_alloc_count() == before
    _lib.check(_call(gpulib, "fricc_seq_cumsum", x, ref))
    torch.cuda.synchronize()
    assert gpulib.fricc_alloc_count() > before
    assert np.array_equal(ref.cpu().numpy().view(np.int64), got.cpu().numpy().view(np.int64))


def test_noalloc_rejects_oversize(gpulib):
    x = torch.zeros(4, dtype=torch.float64, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = gpulib.fricc_seq_cumsum_noalloc(ctypes.c_void_p(x.data_ptr()), MAX_N + 1, ctypes.c_void_p(x.data_ptr()), st)
    assert rc == 1  # FRICC_ERR_ARG, before any device work
    assert b"outside" in gpulib.fricc_last_error()
