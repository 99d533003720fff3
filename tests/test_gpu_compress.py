"""GPU FRI compression against the oracle and the reference's golden vectors:
indices, order and values bit for bit."""
import numpy as np
import pytest
import torch

from conftest import golden

pytestmark = pytest.mark.gpu


def _gpu_sparse(x, m, kind, rn):
    from fricc_gb300 import py_rccsd
    t = py_rccsd.SparseTensor4d(x, x.shape, m, kind, "systematic", rn=rn if kind == "fri" else 0.0)
    flat, vals = t.export()
    idx = np.stack(np.unravel_index(flat, x.shape), axis=1)
    return idx, vals, t


def _same_bits(a, b):
    """Bit-for-bit equality; NaNs compare by position only (CUDA and the host
    CPU generate different NaN payloads for 0/0 and x/NaN)."""
    a, b = np.asarray(a), np.asarray(b)
    na, nb = np.isnan(a), np.isnan(b)
    return np.array_equal(na, nb) and np.array_equal(a[~na].view(np.int64), b[~nb].view(np.int64))


def test_golden_bitexact(gpulib):
    g = golden("compress.npz")
    for k in range(int(g["n_cases"])):
        x = g[f"c{k}_x"]
        m = int(g[f"c{k}_m"])
        for kind in ("fri", "largest"):
            idx, vals, _ = _gpu_sparse(x, m, kind, float(g[f"c{k}_{kind}_rn"]))
            np.testing.assert_array_equal(idx, g[f"c{k}_{kind}_idx"], err_msg=f"case {k} {kind}")
            assert _same_bits(vals, g[f"c{k}_{kind}_val"]), f"case {k} {kind}"


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_mp2_o10v40_vs_oracle(gpulib, oracle, seed):
    """The o10v40 workload (N = 160000, m = 20000), three draws."""
    from fricc_gb300.synthetic import SyntheticSystem
    s = SyntheticSystem(10, 40, 200, 0.05, seed)
    x = s.mp2_amplitudes()[1]
    rn = [0.8401877171547095, 0.3943829268190930, 0.7830992237586059][seed - 1]
    idx, vals, t = _gpu_sparse(x, 20000, "fri", rn)
    ref = oracle.SparseTensor4d(x, x.shape, 20000, "fri", "systematic", rn=rn)
    np.testing.assert_array_equal(idx, ref.idx4)
    assert _same_bits(vals, ref.vals)
    assert t.n_largest() == ref.n_largest


@pytest.mark.parametrize("n,m", [(1, 1), (7, 3), (4096, 100), (4097, 4097), (100_000, 1), (250_000, 60_000),
                                 (300_001, 299_000)])
def test_random_sizes_vs_oracle(gpulib, oracle, n, m):
    rng = np.random.default_rng(n + m)
    x = rng.standard_normal(n) * np.exp(3 * rng.standard_normal(n))
    x = x.reshape(1, 1, 1, n)
    rn = float(rng.random())
    for kind in ("fri", "largest"):
        idx, vals, _ = _gpu_sparse(x, m, kind, rn)
        ref = oracle.SparseTensor4d(x, x.shape, m, kind, "systematic", rn=rn)
        np.testing.assert_array_equal(idx, ref.idx4, err_msg=kind)
        assert _same_bits(vals, ref.vals), kind


def test_ties_zeros_and_degenerate(gpulib, oracle):
    rng = np.random.default_rng(9)
    cases = []
    x = np.round(rng.standard_normal(50_000) * 3)  # many exact ties and zeros
    cases.append((x, 9000))
    x = np.zeros(20_000)
    x[rng.choice(20_000, 300, replace=False)] = rng.standard_normal(300)
    cases.append((x, 1000))  # m > nnz: remaining norm hits 0, samples keep index 0
    x = np.full(10_000, 0.5)  # all equal
    cases.append((x, 777))
    y = rng.standard_normal(30_000)
    y[::3] *= 1e-300  # subnormal and tiny values next to O(1) ones
    cases.append((y, 5000))
    for x, m in cases:
        x = x.reshape(1, 1, 1, -1)
        for rn in (0.0, 0.37, 1.0):
            idx, vals, _ = _gpu_sparse(x, m, "fri", rn)
            ref = oracle.SparseTensor4d(x, x.shape, m, "fri", "systematic", rn=rn)
            np.testing.assert_array_equal(idx, ref.idx4)
            assert _same_bits(vals, ref.vals)


def test_exact_sequential_cumsum(gpulib):
    """fricc_seq_cumsum reproduces a left-to-right FP64 running sum bit for bit
    (numpy's add.accumulate is sequential) on adversarial inputs."""
    import ctypes
    from fricc_gb300 import _lib
    rng = np.random.default_rng(4)
    ulp_half = np.ldexp(1.0, -53)
    cases = [
        rng.random(1_000_003),
        np.exp(40 * rng.standard_normal(200_000)),                  # huge dynamic range
        np.concatenate([np.zeros(5000), rng.random(70_000)]),      # leading zeros
        np.full(300_000, ulp_half),                                 # exact half-ulp ties against 1.0
        np.concatenate([[1.0], np.full(100_000, ulp_half)]),        # ties, parity flips
        np.concatenate([[1.0], np.tile([ulp_half, 3 * ulp_half], 50_000)]),
        np.ldexp(1.0, rng.integers(-1074, -1000, 50_000)).astype(np.float64),  # subnormals
        np.ldexp(1.0, np.arange(0, 200)).astype(np.float64),        # a binade crossing at every step
        rng.random(4096) * 1e-3,
        np.array([3.0]),
    ]
    for k, x in enumerate(cases):
        xd = torch.from_numpy(np.ascontiguousarray(x)).cuda()
        out = torch.empty_like(xd)
        _lib.check(gpulib.fricc_seq_cumsum(ctypes.c_void_p(xd.data_ptr()), xd.numel(),
                                           ctypes.c_void_p(out.data_ptr()),
                                           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
        ref = np.add.accumulate(np.abs(x))
        got = out.cpu().numpy()
        bad = np.flatnonzero(got.view(np.int64) != ref.view(np.int64))
        assert bad.size == 0, f"case {k}: first mismatch at {bad[:3]} {got[bad[:3]]} vs {ref[bad[:3]]}"


def test_errors_raise(gpulib):
    from fricc_gb300 import py_rccsd
    x = np.ones((2, 2, 2, 2))
    with pytest.raises(ValueError):
        py_rccsd.SparseTensor4d(x, x.shape, 17, "fri", "systematic")
    with pytest.raises(ValueError):
        py_rccsd.SparseTensor4d(x, x.shape, 4, "bogus", "systematic")
    with pytest.raises(ValueError):
        py_rccsd.SparseTensor4d(x, x.shape, 4, "fri", "bogus")   # the reference would sample nothing
    with pytest.raises(ValueError):
        py_rccsd.SparseTensor4d(x, x.shape, 0, "fri", "pivotal")
    with pytest.raises(TypeError):
        py_rccsd.SparseTensor4d(x.astype(np.float32), x.shape, 4, "fri", "systematic")


def test_paired_recompress_bit_identical(gpulib):
    """fricc_sp_recompress_pair gives each handle exactly what two separate
    systematic compressions with the same draws give (o20v100: N = 4M)."""
    import ctypes
    import numpy as np
    import torch
    from fricc_gb300 import _lib as L
    from fricc_gb300.synthetic import make_system
    s = make_system("o20v100x64", seed=3)
    t2 = torch.from_numpy(np.ascontiguousarray(s.mp2_amplitudes()[1])).cuda()
    m = 200_000
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    dims = L.i64arr(t2.shape)

    def make(rn):
        h = ctypes.c_void_p()
        L.check(gpulib.fricc_sp_create(ctypes.c_void_p(t2.data_ptr()), dims, m, 0, 0, rn, st, ctypes.byref(h)))
        return h

    def export(h):  # host arrays
        f = np.empty(m, dtype=np.int64)
        v = np.empty(m, dtype=np.float64)
        L.check(gpulib.fricc_sp_export(h, f.ctypes.data_as(ctypes.c_void_p), v.ctypes.data_as(ctypes.c_void_p), st))
        return torch.from_numpy(f), torch.from_numpy(v)

    a, b, c, d = make(0.5), make(0.5), make(0.5), make(0.5)
    L.check(gpulib.fricc_sp_recompress_pair(a, b, ctypes.c_void_p(t2.data_ptr()), 0.123, 0.877, st))
    L.check(gpulib.fricc_sp_recompress(c, ctypes.c_void_p(t2.data_ptr()), 0, 0, 0.123, st))
    L.check(gpulib.fricc_sp_recompress(d, ctypes.c_void_p(t2.data_ptr()), 0, 0, 0.877, st))
    for x, y in ((a, c), (b, d)):
        L.check(gpulib.fricc_sp_status(x))
        fx, vx = export(x)
        fy, vy = export(y)
        assert torch.equal(fx, fy) and torch.equal(vx.view(torch.int64), vy.view(torch.int64))
    fa, _ = export(a)
    fb, _ = export(b)
    assert not torch.equal(fa, fb)  # the draws differ
    rn = torch.tensor([0.31, 0.62], dtype=torch.float64, device="cuda")
    L.check(gpulib.fricc_sp_recompress_pair_dev(a, b, ctypes.c_void_p(t2.data_ptr()), ctypes.c_void_p(rn.data_ptr()),
                                                st))
    L.check(gpulib.fricc_sp_recompress(c, ctypes.c_void_p(t2.data_ptr()), 0, 0, 0.31, st))
    L.check(gpulib.fricc_sp_recompress(d, ctypes.c_void_p(t2.data_ptr()), 0, 0, 0.62, st))
    for x, y in ((a, c), (b, d)):
        fx, vx = export(x)
        fy, vy = export(y)
        assert torch.equal(fx, fy) and torch.equal(vx.view(torch.int64), vy.view(torch.int64))
    for h in (a, b, c, d):
        gpulib.fricc_sp_destroy(h)
    with pytest.raises(ValueError):
        L.check(gpulib.fricc_sp_recompress_pair(a, a, ctypes.c_void_p(t2.data_ptr()), 0.1, 0.2, st))


@pytest.mark.parametrize("compression,method", [("fri", "systematic"), ("fri", "pivotal"), ("largest", "systematic")])
def test_verbose_phase_table(gpulib, oracle, capsys, compression, method):
    """SparseTensor4d(..., verbose=True) prints the reference's phase table
    (src/fri_utils.cpp:509-519): Sorting, P vector, Sampling, Wrap up and
    Total rows, each fraction of the total, the four phases adding up to the
    total; the compression itself is unchanged."""
    from fricc_gb300 import py_rccsd
    from fricc_gb300.rng import GlibcRand
    rng = np.random.default_rng(5)
    x = rng.standard_normal((6, 6, 20, 20)) * rng.random((6, 6, 20, 20)) ** 3
    kw = {"rng": GlibcRand(9)} if method == "pivotal" else {"rn": 0.375}
    quiet = py_rccsd.SparseTensor4d(x, x.shape, 3000, compression, method, False,
                                    **({"rng": GlibcRand(9)} if method == "pivotal" else kw))
    capsys.readouterr()
    loud = py_rccsd.SparseTensor4d(x, x.shape, 3000, compression, method, True, **kw)
    out = capsys.readouterr().out.splitlines()
    assert out[0].split() == ["Subsection", "Fraction", "of", "Total", "Total", "Time"]
    rows = out[2:]
    assert [r[:14].strip() for r in rows] == ["Sorting", "P vector", "Sampling", "Wrap up", "Total"]
    secs = [float(r.split()[-2]) for r in rows]
    fracs = [float(r[14:20]) for r in rows]
    assert secs[4] > 0 and abs(sum(secs[:4]) - secs[4]) <= 1e-3 + 1e-3 * secs[4]
    assert abs(fracs[4] - 1.0) < 1e-9 and all(0.0 <= f <= 1.0001 for f in fracs)
    fq, vq = quiet.export()
    fl, vl = loud.export()
    assert np.array_equal(fq, fl) and np.array_equal(vq.view(np.int64), vl.view(np.int64))
