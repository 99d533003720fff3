"""Pivotal sampling on the GPU (src/fri_utils.cpp:63-127, the binding's default
sampling_method) against the reference's own outputs (tests/golden/pivotal.npz)
and the oracle: indices, values and the number of rand() draws, bit for bit,
with the draws taken from the process's libc rand() (as the reference does)
or from a GlibcRand stream generated on the device."""
import ctypes

import numpy as np
import pytest
import torch

from conftest import golden

pytestmark = pytest.mark.gpu


def test_glibc_uniforms_match_stream(gpulib):
    from fricc_gb300 import _lib as L
    from fricc_gb300.rng import GlibcRand
    for seed, skip, k in ((1, 0, 1), (7, 5, 31), (12345, 100, 1984), (99, 3, 1985), (2024, 17, 50000)):
        g = GlibcRand(seed)
        for _ in range(skip):
            g.rand()
        ref = GlibcRand(seed)
        for _ in range(skip):
            ref.rand()
        want = np.array([ref.uniform() for _ in range(k)])
        out = torch.empty(k, dtype=torch.float64, device="cuda")
        hist, writeback = L.hist_arg(g)
        L.check(gpulib.fricc_glibc_uniforms(hist, k, ctypes.c_void_p(out.data_ptr()),
                                            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
        writeback()
        assert np.array_equal(out.cpu().numpy(), want), (seed, k)
        assert [g.rand() for _ in range(40)] == [ref.rand() for _ in range(40)]


def _cases():
    g = golden("pivotal.npz")
    return g, [k for k in range(int(g["n_cases"])) if int(g[f"c{k}_ok"])]


def test_pivotal_golden_glibc_stream(gpulib):
    from fricc_gb300 import py_rccsd
    from fricc_gb300.rng import GlibcRand
    g, ks = _cases()
    assert len(ks) >= 19
    for k in ks:
        x, m, used, seed = g[f"c{k}_x"], int(g[f"c{k}_m"]), int(g[f"c{k}_used"]), int(g[f"c{k}_seed"])
        r = GlibcRand(seed)
        T = py_rccsd.SparseTensor4d(x, x.shape, m, "fri", "pivotal", rng=r)
        idx = np.array([T.get_element(i)[0] for i in range(m)])
        val = np.array([T.get_element(i)[1] for i in range(m)])
        np.testing.assert_array_equal(idx, g[f"c{k}_idx"], err_msg=f"case {k}")
        assert np.array_equal(val.view(np.int64), g[f"c{k}_val"].view(np.int64)), f"case {k}"
        assert T.draws_used == used
        ref = GlibcRand(seed)
        for _ in range(used):
            ref.rand()
        assert r.rand() == ref.rand()


def test_pivotal_golden_process_rand(gpulib):
    """The default: draws from this process's rand(), exactly as many as the reference."""
    from fricc_gb300 import py_rccsd
    from fricc_gb300.rng import GlibcRand
    libc = ctypes.CDLL(None)
    g, ks = _cases()
    for k in ks[-4:]:
        x, m, used, seed = g[f"c{k}_x"], int(g[f"c{k}_m"]), int(g[f"c{k}_used"]), int(g[f"c{k}_seed"])
        libc.srand(ctypes.c_uint(seed))
        T = py_rccsd.SparseTensor4d(x, x.shape, m)        # compression "fri", sampling "pivotal"
        val = np.array([T.get_element(i)[1] for i in range(m)])
        assert np.array_equal(val.view(np.int64), g[f"c{k}_val"].view(np.int64)), f"case {k}"
        ref = GlibcRand(seed)
        for _ in range(used):
            ref.rand()
        assert libc.rand() == ref.rand()


@pytest.mark.parametrize("o,v,frac,seed", [(20, 100, 0.05, 1), (12, 60, 0.3, 2), (10, 40, 0.01, 3)])
def test_pivotal_large_vs_oracle(gpulib, oracle, o, v, frac, seed):
    """Up to 4M elements: the device chain, draws, decisions and scans against
    the oracle fed the same stream."""
    from fricc_gb300 import _lib as L
    from fricc_gb300.rng import GlibcRand
    from fricc_gb300.synthetic import SyntheticSystem
    s = SyntheticSystem(o, v, 8 * (o + v), 0.05, seed)
    x = np.ascontiguousarray(s.mp2_amplitudes()[1])
    n, m = x.size, max(1, int(frac * x.size))
    # the draws the oracle needs, from the device generator (itself checked above)
    draws = torch.empty(n, dtype=torch.float64, device="cuda")
    gen = GlibcRand(seed)
    h, wb = L.hist_arg(gen)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    L.check(gpulib.fricc_glibc_uniforms(h, n, ctypes.c_void_p(draws.data_ptr()), st))
    oi, ov, ond, oused = oracle.fri_compression_pivotal(x, m, draws=draws.cpu().numpy())
    xd = torch.from_numpy(x).cuda()
    flat = torch.empty(m, dtype=torch.int64, device="cuda")
    vals = torch.empty(m, dtype=torch.float64, device="cuda")
    nd, used = ctypes.c_int64(0), ctypes.c_int64(0)
    r = GlibcRand(seed)
    h2, wb2 = L.hist_arg(r)
    L.check(gpulib.fricc_compress_pivotal(ctypes.c_void_p(xd.data_ptr()), n, m, h2, ctypes.c_void_p(flat.data_ptr()),
                                          ctypes.c_void_p(vals.data_ptr()), ctypes.byref(nd), ctypes.byref(used), st))
    wb2()
    assert used.value == oused and nd.value == ond
    np.testing.assert_array_equal(flat.cpu().numpy(), oi)
    assert np.array_equal(vals.cpu().numpy().view(np.int64), ov.view(np.int64))


def test_pivotal_iteration_vs_oracle(gpulib, oracle):
    """One FRI-CCSD update with pivotal compressions drawing from one GlibcRand
    stream (two compressions in the reference's order) against the oracle."""
    from oracle import ccsd_oracle as CO
    from oracle import pyscf_standin as P
    from fricc_gb300.friccsd import FRICCSDGPU
    from fricc_gb300.rccsd_dense import DeviceERIs
    from fricc_gb300.rng import GlibcRand
    from fricc_gb300.synthetic import SyntheticSystem
    s = SyntheticSystem(6, 24, 120, 0.05, 4)
    settings = {"m_keep": 6000, "compression": "fri", "sampling_method": "pivotal", "verbose": False,
                "compressed_contractions": ["O^2V^4", "O^3V^3", "O^4V^2"]}
    t1, t2 = s.mp2_amplitudes()
    gs = FRICCSDGPU(DeviceERIs.from_system(s), settings, rn_draw=GlibcRand(77))
    gs.update_amps(torch.from_numpy(t1).cuda(), torch.from_numpy(t2).cuda())
    e, _ = gs.read_energy()
    ro = GlibcRand(77)
    eris = P.make_eris(s)
    o1, o2 = CO.update_amps(settings, t1, t2, eris, rn_draw=ro)
    assert abs(e - P.ccsd_energy(o1, o2, eris)) < 1e-10
    assert gs.rn_draw.rand() == ro.rand()   # both streams advanced by the same draws


def test_parallel_sample_golden_one_chunk(gpulib):
    """parallel_sample at one chunk against the reference's own outputs
    (tests/golden/parallel_sample.npz), draws counted."""
    from fricc_gb300 import py_rccsd
    from fricc_gb300.rng import GlibcRand
    g = golden("parallel_sample.npz")
    for k in range(int(g["n_cases"])):
        q, ns, seed, used = g[f"c{k}_q"], int(g[f"c{k}_n"]), int(g[f"c{k}_seed"]), int(g[f"c{k}_used"])
        r = GlibcRand(seed)
        S = py_rccsd.parallel_sample(ns, q, 1, rng=r)
        np.testing.assert_array_equal(S, g[f"c{k}_S"], err_msg=f"case {k}")
        ref = GlibcRand(seed)
        for _ in range(used):
            ref.rand()
        assert r.rand() == ref.rand(), k


@pytest.mark.parametrize("chunks", [2, 5, 16, 128])
def test_parallel_sample_chunks_vs_oracle(gpulib, oracle, chunks):
    """Several chunks (one warp each) against the oracle with the draws in
    chunk order, on an FRI probability vector of 2.6M elements."""
    from fricc_gb300 import py_rccsd
    from fricc_gb300.rng import GlibcRand
    from fricc_gb300.synthetic import SyntheticSystem
    s = SyntheticSystem(18, 90, 864, 0.05, 6)
    x = np.ascontiguousarray(s.mp2_amplitudes()[1]).ravel()
    m = int(0.05 * x.size)
    D, R = oracle.get_d_largest(x, m)
    mp = m - D.size
    q = np.abs(x) / R * float(mp)
    q[D] = 0.0
    r = GlibcRand(chunks)
    S = py_rccsd.parallel_sample(mp, q, chunks, rng=r)
    probe = GlibcRand(chunks)
    draws = np.array([probe.uniform() for _ in range(q.size + chunks + 4)])
    So, used = oracle.parallel_sample(mp, q, chunks, draws)
    np.testing.assert_array_equal(S, So)
    ref = GlibcRand(chunks)
    for _ in range(used):
        ref.rand()
    assert r.rand() == ref.rand()
    assert np.unique(S).size == S.size        # no index twice
