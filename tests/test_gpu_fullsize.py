"""Parity at the benchmark's full sizes.

* The compression of the o30v150 MP2 amplitudes (N = 20.25M, m = 2M) and of
  the o40v200 ones (N = 64M, m = 3.2M), systematic and pivotal, bit for bit
  against the oracle (oracle/fri_oracle.c, pinned to the reference).
* One o30v150 iteration: the float-pair (df64) and FP64 paths from the same
  amplitudes and draws agree to 1e-10 Eh, and a repeated step is bitwise
  identical (deterministic kernels, fixed reduction orders).
* The 2323 contraction at o30v150 (m = 2M, Q = v^2): the float-pair kernel
  against the FP64 kernel, each element to 1e-11 of sum |W||T|
  (the error analysis is beside the assertion)."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _mp2(name):
    from fricc_gb300.synthetic import WORKLOADS, make_system
    s = make_system(name, seed=0)
    return s, WORKLOADS[name]


@pytest.mark.parametrize("name", ["o30v150", "o40v200"])
def test_fullsize_systematic_vs_oracle(gpulib, oracle, name):
    from fricc_gb300 import _lib as L
    from fricc_gb300.rccsd_dense import DeviceERIs
    s, w = _mp2(name)
    E = DeviceERIs.from_system(s)
    o, v = s.nocc, s.nvir
    e = E.mo_energy
    eia = e[:o, None] - e[None, o:]
    t2 = (E.ovov.permute(0, 2, 1, 3) / (eia[:, None, :, None] + eia[None, :, None, :])).contiguous()
    del E
    m, rn = w["m"], 0.6180339887498949
    n = t2.numel()
    flat = torch.empty(m, dtype=torch.int64, device="cuda")
    vals = torch.empty(m, dtype=torch.float64, device="cuda")
    nd = ctypes.c_int64(0)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    L.check(gpulib.fricc_compress(ctypes.c_void_p(t2.data_ptr()), n, m, 0, rn, ctypes.c_void_p(flat.data_ptr()),
                                  ctypes.c_void_p(vals.data_ptr()), ctypes.byref(nd), st))
    x = t2.cpu().numpy().ravel()
    oi, ov, ond = oracle.fri_compression(x, m, rn)
    assert nd.value == ond
    np.testing.assert_array_equal(flat.cpu().numpy(), oi)
    assert np.array_equal(vals.cpu().numpy().view(np.int64), ov.view(np.int64))


def test_fullsize_pivotal_vs_oracle(gpulib, oracle):
    from fricc_gb300 import _lib as L
    from fricc_gb300.rccsd_dense import DeviceERIs
    from fricc_gb300.rng import GlibcRand
    s, w = _mp2("o30v150")
    t2 = torch.from_numpy(np.ascontiguousarray(s.mp2_amplitudes()[1])).cuda()
    m, n = w["m"], t2.numel()
    draws = torch.empty(n, dtype=torch.float64, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    h, _ = L.hist_arg(GlibcRand(5))
    L.check(gpulib.fricc_glibc_uniforms(h, n, ctypes.c_void_p(draws.data_ptr()), st))
    oi, ov, ond, oused = oracle.fri_compression_pivotal(t2.cpu().numpy().ravel(), m, draws=draws.cpu().numpy())
    flat = torch.empty(m, dtype=torch.int64, device="cuda")
    vals = torch.empty(m, dtype=torch.float64, device="cuda")
    nd, used = ctypes.c_int64(0), ctypes.c_int64(0)
    h2, _ = L.hist_arg(GlibcRand(5))
    L.check(gpulib.fricc_compress_pivotal(ctypes.c_void_p(t2.data_ptr()), n, m, h2, ctypes.c_void_p(flat.data_ptr()),
                                          ctypes.c_void_p(vals.data_ptr()), ctypes.byref(nd), ctypes.byref(used), st))
    assert used.value == oused and nd.value == ond
    np.testing.assert_array_equal(flat.cpu().numpy(), oi)
    assert np.array_equal(vals.cpu().numpy().view(np.int64), ov.view(np.int64))


def test_fullsize_iteration_precision_and_determinism(gpulib):
    from fricc_gb300.friccsd import FRICCSDGPU
    from fricc_gb300.rccsd_dense import DeviceERIs
    s, w = _mp2("o30v150")
    E = DeviceERIs.from_system(s)
    t1, t2 = [torch.from_numpy(a).cuda() for a in s.mp2_amplitudes()]
    df = FRICCSDGPU(E, {"m_keep": w["m"]}, precision="df64")
    for _ in range(2):  # away from t1 = 0
        t1, t2 = df.update_amps(t1, t2, rn=[0.25, 0.75])
    a1, a2 = df.update_amps(t1, t2, rn=[0.31, 0.69])
    ea = df.read_energy()[0]
    b1, b2 = df.update_amps(t1, t2, rn=[0.31, 0.69])
    eb = df.read_energy()[0]
    assert ea == eb and torch.equal(a2, b2) and torch.equal(a1, b1)
    fp = FRICCSDGPU(E, {"m_keep": w["m"]}, precision="fp64")
    fp.update_amps(t1, t2, rn=[0.31, 0.69])
    ef = fp.read_energy()[0]
    assert abs(ea - ef) < 1e-10, (ea, ef)


def test_fullsize_2323_pair_vs_fp64(gpulib):
    from fricc_gb300 import _lib as L
    from fricc_gb300 import py_rccsd
    from fricc_gb300.rccsd_dense import DeviceERIs, split_f2
    s, w = _mp2("o30v150")
    E = DeviceERIs.from_system(s)
    o, v = s.nocc, s.nvir
    t2 = torch.from_numpy(np.ascontiguousarray(s.mp2_amplitudes()[1])).cuda()
    T = py_rccsd.SparseTensor4d(t2, t2.shape, w["m"], "fri", "systematic", rn=0.5)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    a = torch.zeros(o * o, v * v, dtype=torch.float64, device="cuda")
    b = torch.zeros_like(a)
    L.check(gpulib.fricc_spmm(T.handle, 0, 1, 2, 3, 1.0, ctypes.c_void_p(E.vvvvT.data_ptr()), v * v,
                              ctypes.c_void_p(a.data_ptr()), st))
    W2 = split_f2(E.vvvvT)
    L.check(gpulib.fricc_spmm_f2(T.handle, 0, 1, 2, 3, 1.0, ctypes.c_void_p(W2.data_ptr()), v * v,
                                 ctypes.c_void_p(b.data_ptr()), st))
    # the pair kernel's error is relative to sum |W||T|, not to the (cancelling)
    # result: c = |T| x |W| through the FP64 kernel (compressing |t2| keeps the
    # same entries, with the absolute values).  Each product carries ~2^-48 of
    # its size; the low word of the running sum is a plain FP32 accumulator
    # (renormalised every 128 terms), whose rounding adds ~2^-45 of the partial
    # sum per term, a random walk over the ~2000 entries of a bucket:
    # ~sqrt(2000) 2^-45 = 1.3e-12 (1.1e-12 measured).  The bound is 1e-11.
    Ta = py_rccsd.SparseTensor4d(t2.abs(), t2.shape, w["m"], "fri", "systematic", rn=0.5)
    c, Wa = torch.zeros_like(a), E.vvvvT.abs()
    L.check(gpulib.fricc_spmm(Ta.handle, 0, 1, 2, 3, 1.0, ctypes.c_void_p(Wa.data_ptr()), v * v,
                              ctypes.c_void_p(c.data_ptr()), st))
    torch.cuda.synchronize()
    assert bool(((a - b).abs() <= 1e-11 * c + 1e-300).all()), float(((a - b).abs() / c.clamp_min(1e-300)).max())
