"""The eleven contraction terms on the GPU against the oracle (same nonzero
order per output element; the GPU fuses each multiply-add, so the bound is
a relative tolerance, not bit equality) and against the golden outputs of
the reference's own contract_DTSpT.  Also the reference's own test pattern:
each term equals np.einsum on a "largest"-compressed sparse T2."""
import numpy as np
import pytest
import torch

from conftest import golden

pytestmark = pytest.mark.gpu

TERMS = ("0101", "2323", "1302", "1202", "1303", "1203", "1323", "0112", "0113", "0313", "0312")
W_SHAPE = {"0101": "oooo", "2323": "vvvv", "1302": "voov", "1202": "vovo", "1303": "voov", "1203": "vovo",
           "1323": "ovov", "0112": "ovov", "0113": "ovov", "0313": "ovov", "0312": "ovov"}
OUT_SHAPE = {"1323": "oooo", "0112": "voov", "0113": "voov", "0313": "voov", "0312": "vovo"}
EINSUM = {"0101": ("klij,klab->ijab", 1.0), "2323": ("abcd,ijcd->ijab", 1.0), "1302": ("akic,kjcb->ijab", 2.0),
          "1202": ("akci,kjcb->ijab", -1.0), "1303": ("akic,kjbc->ijab", 1.0), "1203": ("bkci,kjac->ijab", 1.0),
          "1323": ("kcld,ijcd->klij", 1.0), "0112": ("ldkc,ilda->akic", -0.5), "0113": ("ldkc,ilad->akic", 1.0),
          "0313": ("lckd,ilad->akic", -0.5), "0312": ("lckd,ilda->akci", -0.5)}
RTOL = 1e-12  # relative to the largest |output| of the term


def _close(a, b, rtol=RTOL):
    scale = max(np.abs(b).max(), 1.0)
    assert np.abs(a - b).max() <= rtol * scale, np.abs(a - b).max() / scale


def test_golden(gpulib):
    from fricc_gb300 import py_rccsd
    g = golden("contract.npz")
    for si in range(3):
        t2 = g[f"s{si}_t2"]
        T = py_rccsd.SparseTensor4d(t2, t2.shape, int(g[f"s{si}_m"]), "largest")
        for term in TERMS:
            W = g[f"s{si}_{term}_W"]
            for strided in (0, 1):
                Wuse = W if not strided else np.ascontiguousarray(W.transpose(3, 2, 1, 0)).transpose(3, 2, 1, 0)
                out = g[f"s{si}_{term}_init"].copy()
                py_rccsd.contract_DTSpT(Wuse, T, out, term)
                _close(out, g[f"s{si}_{term}_out{strided}"])


@pytest.mark.parametrize("no,nv,frac", [(4, 8, 0.1), (5, 10, 0.01), (10, 20, 0.001), (7, 31, 0.3)])
def test_einsum_pattern(gpulib, no, nv, frac):
    """fricc/tests/test_sparse_tensors.py: term(W, largest-compressed T) == einsum(W, T)."""
    from fricc_gb300 import py_rccsd
    rng = np.random.default_rng(int(no * 100 + nv))
    d = {"o": no, "v": nv}
    t2 = np.zeros(no * no * nv * nv)
    nnz = max(1, int(t2.size * frac))
    t2[rng.choice(t2.size, nnz, replace=False)] = rng.random(nnz)
    t2 = t2.reshape(no, no, nv, nv)
    T = py_rccsd.SparseTensor4d(t2, t2.shape, nnz, "largest")
    for term in TERMS:
        W = rng.random(tuple(d[c] for c in W_SHAPE[term]))
        spec, coef = EINSUM[term]
        ref = coef * np.einsum(spec, W, t2)
        out = np.zeros(ref.shape)
        py_rccsd.contract_DTSpT(W, T, out, term)
        _close(out, ref)


def test_vs_oracle_fri_tensor_and_device_views(gpulib, oracle):
    """A FRI-compressed MP2 T2 (o10v40 sizes), W and out as torch CUDA views
    with permuted strides, accumulated in place on top of nonzero data."""
    from fricc_gb300 import py_rccsd
    from fricc_gb300.synthetic import SyntheticSystem
    s = SyntheticSystem(10, 40, 200, 0.05, 4)
    x = s.mp2_amplitudes()[1]
    rn = 0.25
    T = py_rccsd.SparseTensor4d(x, x.shape, 20000, "fri", "systematic", rn=rn)
    To = oracle.SparseTensor4d(x, x.shape, 20000, "fri", "systematic", rn=rn)
    rng = np.random.default_rng(0)
    d = {"o": 10, "v": 40}
    for term in TERMS:
        W = rng.standard_normal(tuple(d[c] for c in W_SHAPE[term]))
        out0 = rng.standard_normal(tuple(d[c] for c in OUT_SHAPE.get(term, "oovv")))
        ref = out0.copy()
        oracle.contract_DTSpT(W, To, ref, term)
        # device tensors stored transposed, passed as (W-shaped) strided views
        Wd = torch.from_numpy(np.ascontiguousarray(W.transpose(2, 0, 3, 1))).cuda().permute(1, 3, 0, 2)
        Od = torch.from_numpy(np.ascontiguousarray(out0.transpose(3, 1, 0, 2))).cuda().permute(2, 1, 3, 0)
        py_rccsd.contract_DTSpT(Wd, T, Od, term)
        _close(Od.cpu().numpy(), ref)


def test_deterministic(gpulib):
    from fricc_gb300 import py_rccsd
    rng = np.random.default_rng(1)
    x = rng.standard_normal((6, 6, 30, 30))
    T = py_rccsd.SparseTensor4d(x, x.shape, 5000, "fri", "systematic", rn=0.5)
    W = rng.standard_normal((30, 30, 30, 30))
    outs = []
    for _ in range(3):
        o = np.zeros((6, 6, 30, 30))
        py_rccsd.contract_DTSpT(W, T, o, "2323")
        outs.append(o)
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[1], outs[2])


def test_bad_shapes_raise(gpulib):
    from fricc_gb300 import py_rccsd
    x = np.random.default_rng(2).standard_normal((3, 3, 5, 5))
    T = py_rccsd.SparseTensor4d(x, x.shape, 20, "largest")
    with pytest.raises(ValueError):
        py_rccsd.contract_DTSpT(np.zeros((5, 5, 5, 4)), T, np.zeros((3, 3, 5, 5)), "2323")
    with pytest.raises(ValueError):
        py_rccsd.contract_DTSpT(np.zeros((5, 5, 5, 5)), T, np.zeros((3, 3, 5, 5)), "9999")


def test_spmm_f2_matches_fp64(gpulib):
    """The FP32-pair kernel against the FP64 kernel on the same generic SpMM
    (o10v40-sized sparse tensor, 2323 layout and an O^3V^3 layout)."""
    import ctypes
    from fricc_gb300 import _lib, py_rccsd
    from fricc_gb300.rccsd_dense import split_f2
    rng = np.random.default_rng(3)
    o, v = 10, 40
    x = rng.standard_normal((o, o, v, v)) * np.exp(rng.standard_normal((o, o, v, v)))
    T = py_rccsd.SparseTensor4d(x, x.shape, 20000, "fri", "systematic", rn=0.6)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    cases = ((0, 1, 2, 3, v * v, v * v), (1, 3, 0, 2, o * v, o * v), (3, 0, 1, 2, o * v, o * v),
             (0, 1, 2, 3, v * v, 777), (2, 3, 0, 1, o * o, 1), (2, 3, 0, 1, o * o, 2049))   # odd / tiny / ragged QS
    for (pa, pb, ka, kb, nkey, QS) in cases:
        W = torch.from_numpy(rng.standard_normal((nkey, QS)) * 10.0 ** rng.integers(-6, 2, (nkey, 1))).cuda()
        nP = {0: o, 1: o, 2: v, 3: v}[pa] * {0: o, 1: o, 2: v, 3: v}[pb]
        out0 = torch.from_numpy(rng.standard_normal((nP, QS))).cuda()
        a, b = out0.clone(), out0.clone()
        _lib.check(gpulib.fricc_spmm(T.handle, pa, pb, ka, kb, -0.5, ctypes.c_void_p(W.data_ptr()), QS,
                                     ctypes.c_void_p(a.data_ptr()), st))
        W2 = split_f2(W, QS)
        _lib.check(gpulib.fricc_spmm_f2(T.handle, pa, pb, ka, kb, -0.5, ctypes.c_void_p(W2.data_ptr()), QS,
                                        ctypes.c_void_p(b.data_ptr()), st))
        a, b = a.cpu().numpy(), b.cpu().numpy()
        # per-element error relative to the sum of |terms| is ~1e-14; compare to the output scale
        assert np.abs(a - b).max() <= 1e-12 * np.abs(a).max(), np.abs(a - b).max() / np.abs(a).max()


def test_split_f2_bits_bound_and_edges(gpulib):
    """The integer float-pair split: |x - hi - lo| < 2^-47 |x| across the fast
    range 2^-74 <= |x| < 2^128, exact-float inputs give lo = 0, and zeros,
    tiny, huge, infinite and NaN inputs follow the conversion path."""
    from fricc_gb300.rccsd_dense import split_f2
    rng = np.random.default_rng(9)
    e = rng.integers(-74, 128, 100000)
    x = rng.choice([-1.0, 1.0], e.size) * rng.uniform(1.0, 2.0, e.size) * np.exp2(e.astype(np.float64))
    x[::7] = x[::7].astype(np.float32).astype(np.float64)
    edge = np.array([0.0, -0.0, 2.0**-74, -2.0**-74, 2.0**-75, 2.0**127 * 1.99, 2.0**128, 1e-300, 5e-324,
                     np.inf, -np.inf, np.nan, 1.0, -1.0 - 2.0**-52])
    xs = np.concatenate([x, edge])
    xs = np.concatenate([xs, [0.0]]) if xs.size % 2 else xs
    out = split_f2(torch.from_numpy(xs).cuda().view(1, 1, -1), qs=xs.size).cpu().numpy().reshape(-1, 4)
    hi = np.stack([out[:, 0], out[:, 1]], 1).reshape(-1).astype(np.float64)
    lo = np.stack([out[:, 2], out[:, 3]], 1).reshape(-1).astype(np.float64)
    n = x.size
    err = np.abs(hi[:n] + lo[:n] - x) / np.abs(x)
    assert err.max() < 2.0**-47
    assert np.all(lo[:n][::7] == 0.0)
    with np.errstate(invalid="ignore", over="ignore"):
        want_hi = edge.astype(np.float32).astype(np.float64)
        want_lo = (edge - want_hi).astype(np.float32).astype(np.float64)
    for k, v in enumerate(edge):
        h, l = hi[n + k], lo[n + k]
        if np.isnan(v):
            assert np.isnan(h)
        elif v == 0.0 or not np.isfinite(v) or abs(v) < 2.0**-74 or abs(v) >= 2.0**128:
            assert h == want_hi[k] and (l == want_lo[k] or (np.isnan(l) and np.isnan(want_lo[k]))), (v, h, l)
        else:
            assert abs(h + l - v) <= 2.0**-47 * abs(v), v


@pytest.mark.parametrize("perm", [(0, 1, 2, 3), (2, 0, 3, 1), (2, 0, 1, 3), (1, 0, 2, 3)])
@pytest.mark.parametrize("o,v", [(4, 37), (6, 64)])
def test_sym_add_matches_torch(gpulib, perm, o, v):
    """out += c (X + X^T(0,1,3,2)) in one pass, for the strided views the
    iteration passes (and odd nvir: partial 32 x 32 tiles)."""
    import torch
    from fricc_gb300.rccsd_dense import sym_add
    g = torch.Generator().manual_seed(9)
    # base laid out so that base.permute(perm) has shape (o, o, v, v)
    shape = [0, 0, 0, 0]
    for k, p in enumerate(perm):
        shape[p] = (o, o, v, v)[k]
    base = torch.randn(*shape, generator=g, dtype=torch.float64).cuda()
    X = base.permute(*perm)
    out = torch.randn(o, o, v, v, generator=g, dtype=torch.float64).cuda()
    ref = out + -0.5 * (X + X.permute(1, 0, 3, 2))
    sym_add(out, X, -0.5)
    torch.testing.assert_close(out, ref, rtol=0, atol=0)


def test_batch_entry_points_match_single_calls(gpulib):
    """fricc_sp_recompress_batch and fricc_contract_batch: every item is bit
    for bit its single-handle call (same kernels, issued in order)."""
    import ctypes

    from fricc_gb300 import _lib, py_rccsd
    rng = np.random.default_rng(5)
    o, v, m, R = 4, 9, 300, 2
    dims = (o, o, v, v)
    Ts = [py_rccsd.SparseTensor4d(rng.standard_normal(dims), dims, m, "fri", "systematic", rn=0.3) for _ in range(R)]
    new = [torch.from_numpy(rng.standard_normal(dims)).cuda() for _ in range(R)]
    rns = (ctypes.c_double * R)(0.11, 0.77)
    hs = (ctypes.c_void_p * R)(*[T.handle.value for T in Ts])
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(gpulib.fricc_sp_recompress_batch(R, hs, (ctypes.c_void_p * R)(*[x.data_ptr() for x in new]), 0, 0,
                                                rns, st))
    for r in range(R):
        ref = py_rccsd.SparseTensor4d(new[r], dims, m, "fri", "systematic", rn=rns[r])
        (fa, va), (fb, vb) = Ts[r].export(), ref.export()
        assert np.array_equal(fa, fb) and np.array_equal(va.view(np.int64), vb.view(np.int64)), r
    Ws = [torch.from_numpy(rng.standard_normal((v, v, v, v))).cuda() for _ in range(R)]
    outs = [torch.from_numpy(rng.standard_normal(dims)).cuda() for _ in range(R)]
    refs = [x.clone() for x in outs]
    cat = lambda ts, f: _lib.i64arr([k for t in ts for k in f(t)])  # noqa: E731
    _lib.check(gpulib.fricc_contract_batch(
        b"2323", R, (ctypes.c_void_p * R)(*[w.data_ptr() for w in Ws]), cat(Ws, lambda t: t.shape),
        cat(Ws, lambda t: t.stride()), hs, (ctypes.c_void_p * R)(*[x.data_ptr() for x in outs]),
        cat(outs, lambda t: t.shape), cat(outs, lambda t: t.stride()), st))
    for r in range(R):
        py_rccsd.contract_DTSpT(Ws[r], Ts[r], refs[r], "2323")
        assert torch.equal(outs[r], refs[r]), r
