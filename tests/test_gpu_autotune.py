"""Autotuned launch configurations: the sparse kernel's output pairs per
thread and the compression's select-digit width change no result bit; a
tuned df64 iteration (GEMM tiles and splits, sparse kernel, compression
schedule) agrees with the untuned one to rounding (the GEMM tile and split
order its sums)."""
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
    # pairs per thread, each as a grid launch (knob 5 unset) and as the
    # persistent q-tile-major launch at 1, 3 and 8 CTAs per SM
    for ppt in (1, 2, 4):
        for persist in (-1, 1, 3, 8):
            L.check(gpulib.fricc_tune_set(0, ppt))
            L.check(gpulib.fricc_tune_set(5, persist))
            o_ = torch.zeros(o * o, QS, dtype=torch.float64, device="cuda")
            L.check(gpulib.fricc_spmm_f2(T.handle, 0, 1, 2, 3, 1.0, ctypes.c_void_p(W2.data_ptr()), QS,
                                         ctypes.c_void_p(o_.data_ptr()), st))
            outs.append(o_)
    L.check(gpulib.fricc_tune_set(0, -1))
    L.check(gpulib.fricc_tune_set(5, -1))
    assert all(torch.equal(outs[0], x) for x in outs[1:])


@pytest.mark.parametrize("shape,m", [((8, 8, 40, 40), 20000), ((12, 12, 50, 50), 90000)])
def test_select_digit_width_keeps_the_same_entries(gpulib, oracle, shape, m):
    """The top-m selection schedule (the first select digit's width, 10-13
    bits) changes how many candidates the exact sort takes, never the
    compression: single and batched compressions at every width keep the
    oracle's entries bit for bit."""
    from fricc_gb300 import _lib as L
    from fricc_gb300.friccsd import _Handle
    rng = np.random.default_rng(5)
    x_h = rng.standard_normal((2,) + shape) * rng.random((2,) + shape) ** 4
    x = torch.from_numpy(x_h).cuda()
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    refs = [[oracle.SparseTensor4d(x_h[r], shape, m, "fri", "systematic", rn=rn) for rn in (0.3, 0.7)]
            for r in range(2)]
    rn = torch.tensor([[0.3, 0.7], [0.3, 0.7]], dtype=torch.float64, device="cuda")
    spb = ctypes.c_void_p()
    L.check(gpulib.fricc_spb_create(2, L.i64arr(shape), m, st, ctypes.byref(spb)))
    flat = np.empty(m, dtype=np.int64)
    vals = np.empty(m, dtype=np.float64)
    try:
        for bits in (10, 11, 12, 13):
            L.check(gpulib.fricc_tune_set(4, bits))
            h = _Handle()
            h.compress(x[0], m, "fri", 0.3, st)
            L.check(gpulib.fricc_sp_status(h.h))
            L.check(gpulib.fricc_sp_export(h.h, ctypes.c_void_p(flat.ctypes.data), ctypes.c_void_p(vals.ctypes.data),
                                           st))
            assert np.array_equal(flat, refs[0][0].flat), bits
            assert np.array_equal(vals.view(np.int64), refs[0][0].vals.view(np.int64)), bits
            h.free()
            L.check(gpulib.fricc_spb_recompress_pair(spb, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(rn.data_ptr()),
                                                     st))
            L.check(gpulib.fricc_spb_status(spb, None))
            for r in range(2):
                for which in (0, 1):
                    L.check(gpulib.fricc_spb_export(spb, which, r, ctypes.c_void_p(flat.ctypes.data),
                                                    ctypes.c_void_p(vals.ctypes.data), st))
                    assert np.array_equal(flat, refs[r][which].flat), (bits, r, which)
                    assert np.array_equal(vals.view(np.int64), refs[r][which].vals.view(np.int64)), (bits, r, which)
    finally:
        L.check(gpulib.fricc_tune_set(4, -1))
        gpulib.fricc_spb_destroy(spb)


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
    assert any(k[0] == "compress_pair" for k in a._tuner.best)
    # replays are deterministic
    c1, c2 = a.update_amps(t1, t2, rn=[0.5, 0.5])
    d1, d2 = a.update_amps(t1, t2, rn=[0.5, 0.5])
    assert torch.equal(c2, d2) and torch.equal(c1, d1)
