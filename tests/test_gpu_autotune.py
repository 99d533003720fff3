"""Autotuned launch configurations: the sparse kernel's output pairs per
thread change no result bit; a tuned df64 iteration agrees with the
untuned one to rounding (the GEMM tile and split order its sums)."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_spmm_ppt_knob_bit_identical(gpulib):
    from fricc_gb300 import _lib as L
    from fricc_gb300 import py_rccsd
    from fricc_gb300.rccsd_dense import split_f2
    from fricc_gb300.synthetic import make_system
    s = make_system("o10v40", seed=1)
    o, v = s.nocc, s.nvir
    t2 = torch.from_numpy(np.ascontiguousarray(s.mp2_amplitudes()[1])).cuda()
    T = py_rccsd.SparseTensor4d(t2, t2.shape, 20000, "fri", "systematic", rn=0.3)
    W = torch.randn(v * v, v * v + 3, dtype=torch.float64, device="cuda")  # odd QS: a partial q tile
    QS = v * v + 3
    W2 = split_f2(W, QS)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    outs = []
    for ppt in (1, 2, 4):
        L.check(gpulib.fricc_tune_set(0, ppt))
        o_ = torch.zeros(o * o, QS, dtype=torch.float64, device="cuda")
        L.check(gpulib.fricc_spmm_f2(T.handle, 0, 1, 2, 3, 1.0, ctypes.c_void_p(W2.data_ptr()), QS,
                                     ctypes.c_void_p(o_.data_ptr()), st))
        outs.append(o_)
    L.check(gpulib.fricc_tune_set(0, -1))
    assert torch.equal(outs[0], outs[1]) and torch.equal(outs[1], outs[2])


def test_autotuned_iteration_matches(gpulib):
    from fricc_gb300.friccsd import FRICCSDGPU
    from fricc_gb300.rccsd_dense import DeviceERIs
    from fricc_gb300.synthetic import make_system
    s = make_system("o10v40", seed=0)
    E = DeviceERIs.from_system(s)
    t1, t2 = [torch.from_numpy(x).cuda() for x in s.mp2_amplitudes()]
    a = FRICCSDGPU(E, {"m_keep": 20000}, precision="df64", autotune=True)
    b = FRICCSDGPU(E, {"m_keep": 20000}, precision="df64")
    for it in range(3):
        rn = [0.2 + 0.2 * it, 0.55]
        a1, a2 = a.update_amps(t1, t2, rn=rn)
        b1, b2 = b.update_amps(t1, t2, rn=rn)
        assert abs(a.read_energy()[0] - b.read_energy()[0]) < 1e-14
        torch.testing.assert_close(a2, b2, rtol=1e-12, atol=1e-16)
        t1, t2 = a1, a2
    assert a._tuner.best and a._tuner.tuning_s > 0
    # replays are deterministic
    c1, c2 = a.update_amps(t1, t2, rn=[0.5, 0.5])
    d1, d2 = a.update_amps(t1, t2, rn=[0.5, 0.5])
    assert torch.equal(c2, d2) and torch.equal(c1, d1)
