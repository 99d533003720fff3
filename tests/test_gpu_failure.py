"""Failure paths, exercised without faulting the GPU.

* The iteration loop's aborts (fricc/friccsd.py:444-453): amplitudes
  poisoned on the host with a NaN, or blown up, stop FRICCSDGPU.kernel with
  conv = False at the same iteration as the oracle's loop.
* A bounded device wait that runs out: with the test knob set, one tile of
  the compression's compaction polls a word nothing sets and gives up; the
  compression reports FRICC_ERR_TIMEOUT through its status, the context
  stays usable, and the next compression on the same handle succeeds bit
  for bit."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SETTINGS = {"compression": "fri", "sampling_method": "systematic", "verbose": False,
            "compressed_contractions": ["O^2V^4", "O^3V^3", "O^4V^2"]}


def _system():
    from fricc_gb300.synthetic import SyntheticSystem
    return SyntheticSystem(6, 24, 120, 0.05, 3)


def _both_loops(t1, t2, m, draws):
    from fricc_gb300.friccsd import FRICCSDGPU
    from fricc_gb300.rccsd_dense import DeviceERIs
    from oracle import ccsd_oracle as CO
    from oracle import pyscf_standin as P
    s = _system()
    it_g = iter(draws)
    gs = FRICCSDGPU(DeviceERIs.from_system(s), dict(SETTINGS, m_keep=m), rn_draw=lambda: next(it_g))
    conv_g, e_g, _, _, en_g = gs.kernel(torch.from_numpy(t1).cuda(), torch.from_numpy(t2).cuda(), max_cycle=6)
    it_o = iter(draws)
    conv_o, e_o, _, _, en_o = CO.kernel(dict(SETTINGS, m_keep=m), P.make_eris(s), t1.copy(), t2.copy(),
                                        max_cycle=6, rn_draw=lambda: next(it_o))
    return (conv_g, e_g, en_g), (conv_o, e_o, en_o)


def test_nan_amplitudes_stop_the_loop(gpulib, oracle):
    t1, t2 = _system().mp2_amplitudes()
    t2 = t2.copy()
    t2[1, 2, 3, 4] = np.nan
    draws = [0.25 + 0.05 * k for k in range(12)]
    (conv_g, e_g, en_g), (conv_o, e_o, en_o) = _both_loops(t1, t2, 3000, draws)
    assert conv_g is False and conv_o is False
    assert len(en_g) == len(en_o) == 1 and np.isnan(e_g) and np.isnan(e_o)


def test_blown_up_amplitudes_stop_the_loop(gpulib, oracle):
    t1, t2 = _system().mp2_amplitudes()
    t2 = t2 * 1e5   # the loop runs away: |dE| passes 1e5 Eh at the third iteration
    draws = [0.25 + 0.05 * k for k in range(12)]
    (conv_g, e_g, en_g), (conv_o, e_o, en_o) = _both_loops(t1, t2, 3000, draws)
    assert conv_g is False and conv_o is False
    assert len(en_g) == len(en_o) == 3
    assert abs(en_g[-1] - en_g[-2]) > 1e5
    assert np.allclose(en_g, en_o, rtol=1e-9, atol=0.0)


def test_bounded_wait_runs_out_and_the_context_stays_usable(gpulib, oracle):
    from fricc_gb300 import _lib as L
    from fricc_gb300.friccsd import _Handle
    rng = np.random.default_rng(21)
    x_h = rng.standard_normal((8, 8, 40, 40)) * rng.random((8, 8, 40, 40)) ** 4
    x = torch.from_numpy(x_h).cuda()
    m = 20000
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    h = _Handle()
    L.check(gpulib.fricc_tune_set(3, 2000))   # knob 3: the test-only wait of 2000 polls
    try:
        h.compress(x, m, "fri", 0.5, st)
        with pytest.raises(L.FriccError) as ex:
            L.check(gpulib.fricc_sp_status(h.h))
        assert ex.value.status == 5            # FRICC_ERR_TIMEOUT
    finally:
        L.check(gpulib.fricc_tune_set(3, -1))
    h.compress(x, m, "fri", 0.5, st)           # the same handle, re-compressed
    L.check(gpulib.fricc_sp_status(h.h))
    flat = np.empty(m, dtype=np.int64)
    vals = np.empty(m, dtype=np.float64)
    L.check(gpulib.fricc_sp_export(h.h, ctypes.c_void_p(flat.ctypes.data), ctypes.c_void_p(vals.ctypes.data), st))
    ref = oracle.SparseTensor4d(x_h, x_h.shape, m, "fri", "systematic", rn=0.5)
    assert np.array_equal(flat, ref.flat)
    assert np.array_equal(vals.view(np.int64), ref.vals.view(np.int64))
    h.free()
