"""The split-precision form: integral blocks rebuilt from the BF16 hi + lo
Cholesky factor on the tcgen05 tensor cores (fricc_gb300.cholesky), the
O^2V^4 term against the FP32 (vv|vv) block (fricc_spmm_f1), and the
iteration's |dE_corr| against the plain FP64 GPU path (bound 1e-6 Eh)."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def systems():
    from fricc_gb300.cholesky import split_eris
    from fricc_gb300.rccsd_dense import DeviceERIs
    from fricc_gb300.synthetic import make_system
    s = make_system("o10v40", seed=0)
    return s, DeviceERIs.from_system(s), split_eris(s)


def test_split_blocks(gpulib, systems):
    s, E, Es = systems
    Lf = torch.from_numpy(s.L).cuda()
    o = s.nocc
    La = Lf.abs()
    for name in ("ovvv", "oovv"):
        sl = {"o": slice(0, o), "v": slice(o, s.nmo)}
        p, q, r, t = (sl[c] for c in name)
        scale = torch.einsum("Ppq,Prs->pqrs", La[:, p, q], La[:, r, t])
        err = float(((getattr(Es, name) - getattr(E, name)).abs() / scale).max())
        assert err < 2.0 ** -14, (name, err)
    for name in ("oooo", "ovoo", "ovov", "ovvo"):  # FP32-pair GEMM: ~2^-40 of sum |L||L|
        sl = {"o": slice(0, o), "v": slice(o, s.nmo)}
        p, q, r, t = (sl[c] for c in name)
        scale = torch.einsum("Ppq,Prs->pqrs", La[:, p, q], La[:, r, t])
        assert float(((getattr(Es, name) - getattr(E, name)).abs() / scale).max()) < 1e-11, name
    torch.testing.assert_close(Es.S0, E.S0, rtol=1e-12, atol=1e-15)
    assert Es.vvvvT is None


def test_spmm_f1_matches_fp64_kernel(gpulib, systems):
    from fricc_gb300 import _lib as L
    from fricc_gb300 import py_rccsd
    s, E, Es = systems
    o, v = s.nocc, s.nvir
    R = Es.vvvv_rebuild
    W = R.rebuild()
    R.check()
    t2 = torch.from_numpy(np.ascontiguousarray(s.mp2_amplitudes()[1])).cuda()
    T = py_rccsd.SparseTensor4d(t2, t2.shape, 20000, "fri", "systematic", rn=0.5)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    W64 = W[:, : v * v].double().contiguous()
    a = torch.randn(o * o, v * v, dtype=torch.float64, device="cuda") * 1e-3
    b = a.clone()
    L.check(gpulib.fricc_spmm(T.handle, 0, 1, 2, 3, 1.0, ctypes.c_void_p(W64.data_ptr()), v * v,
                              ctypes.c_void_p(a.data_ptr()), st))
    L.check(gpulib.fricc_spmm_f1(T.handle, 0, 1, 2, 3, 1.0, ctypes.c_void_p(W.data_ptr()), v * v, R.ldw,
                                 ctypes.c_void_p(b.data_ptr()), st))
    Ta = py_rccsd.SparseTensor4d(t2.abs(), t2.shape, 20000, "fri", "systematic", rn=0.5)
    c = torch.zeros_like(a)
    Wa = W64.abs()
    L.check(gpulib.fricc_spmm(Ta.handle, 0, 1, 2, 3, 1.0, ctypes.c_void_p(Wa.data_ptr()), v * v,
                              ctypes.c_void_p(c.data_ptr()), st))
    torch.cuda.synchronize()
    bound = 1e-11 * (c + 1e-3 * 4)  # sum |W||T| plus the initial output's scale
    assert bool(((a - b).abs() <= bound).all())


def test_spmm_f32_within_fp32_error(gpulib, systems):
    """The plain-FP32 sparse kernel: each output within 2^-16 of sum |W||T|
    of the FP64 kernel's (FP32 products and an FP32 sum over a bucket)."""
    from fricc_gb300 import _lib as L
    from fricc_gb300 import py_rccsd
    s, E, Es = systems
    o, v = s.nocc, s.nvir
    R = Es.vvvv_rebuild
    W = R.rebuild()
    t2 = torch.from_numpy(np.ascontiguousarray(s.mp2_amplitudes()[1])).cuda()
    T = py_rccsd.SparseTensor4d(t2, t2.shape, 20000, "fri", "systematic", rn=0.5)
    Ta = py_rccsd.SparseTensor4d(t2.abs(), t2.shape, 20000, "fri", "systematic", rn=0.5)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    W64 = W[:, : v * v].double().contiguous()
    Wa = W64.abs()
    a = torch.randn(o * o, v * v, dtype=torch.float64, device="cuda") * 1e-3
    b, c = a.clone(), torch.zeros_like(a)
    L.check(gpulib.fricc_spmm(T.handle, 0, 1, 2, 3, 1.0, ctypes.c_void_p(W64.data_ptr()), v * v,
                              ctypes.c_void_p(a.data_ptr()), st))
    L.check(gpulib.fricc_spmm_f32(T.handle, 0, 1, 2, 3, 1.0, ctypes.c_void_p(W.data_ptr()), v * v, R.ldw,
                                  ctypes.c_void_p(b.data_ptr()), st))
    L.check(gpulib.fricc_spmm(Ta.handle, 0, 1, 2, 3, 1.0, ctypes.c_void_p(Wa.data_ptr()), v * v,
                              ctypes.c_void_p(c.data_ptr()), st))
    torch.cuda.synchronize()
    assert bool(((a - b).abs() <= 2.0 ** -16 * c + 1e-18).all())


def test_dense_spmm_and_split_b_rebuild(gpulib, systems):
    """The split form's dense path: the (vv|vv) rebuild written as the B'
    operand (hi + lo within 2^-16 of (ac|bd)), and the compressed T densified
    and contracted on the tensor cores against it, within 2^-14 of
    sum |W||T| of the FP64 sparse kernel."""
    from fricc_gb300 import _lib as L
    from fricc_gb300 import py_rccsd
    from fricc_gb300.cholesky import dense_spmm
    s, E, Es = systems
    o, v = s.nocc, s.nvir
    R = Es.vvvv_rebuild
    Bt = R.rebuild_split_b()
    R.check()
    vv = v * v
    hi, lo = Bt[:, :vv].double(), Bt[:, vv:2 * vv].double()
    assert torch.equal(Bt[:, :vv], Bt[:, 2 * vv:3 * vv]) and bool((Bt[:, 3 * vv:] == 0).all())
    ref = E.vvvvT.reshape(vv, vv).T  # [q=(a,b)][k=(c,d)] = (ac|bd)
    Lv = torch.from_numpy(s.L).cuda()[:, o:, o:].abs()
    scale = torch.einsum("Pac,Pbd->abcd", Lv, Lv).reshape(vv, vv)
    assert float(((hi + lo - ref).abs() / scale).max()) < 2.0 ** -14
    t2 = torch.from_numpy(np.ascontiguousarray(s.mp2_amplitudes()[1])).cuda()
    T = py_rccsd.SparseTensor4d(t2, t2.shape, 20000, "fri", "systematic", rn=0.5)
    Ta = py_rccsd.SparseTensor4d(t2.abs(), t2.shape, 20000, "fri", "systematic", rn=0.5)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    a = torch.randn(o * o, vv, dtype=torch.float64, device="cuda") * 1e-3
    b, c = a.clone(), torch.zeros_like(a)
    W = E.vvvvT.reshape(vv, vv).contiguous()
    L.check(gpulib.fricc_spmm(T.handle, 0, 1, 2, 3, 1.0, ctypes.c_void_p(W.data_ptr()), vv,
                              ctypes.c_void_p(a.data_ptr()), st))
    assert dense_spmm(T.handle, t2.shape, 0, 1, 2, 3, 1.0, Bt, vv, b)
    Wa = scale.T.contiguous()  # [k][q] bound of |W|
    L.check(gpulib.fricc_spmm(Ta.handle, 0, 1, 2, 3, 1.0, ctypes.c_void_p(Wa.data_ptr()), vv,
                              ctypes.c_void_p(c.data_ptr()), st))
    torch.cuda.synchronize()
    assert bool(((a - b).abs() <= 2.0 ** -14 * c + 1e-18).all())


@pytest.mark.parametrize("o,v", [(3, 17), (4, 40), (5, 80), (6, 131)])
def test_split_b_rebuild_triangle(gpulib, o, v):
    """The (vv|vv) rebuild into the B' operand runs only the upper-triangle
    tiles of its symmetric GEMM and mirrors them: every element of a
    NaN-filled output is written, B'[(a,b)][(c,d)] equals B'[(b,a)][(d,c)]
    bit for bit (both written from one computed value), hi + lo is within
    2^-14 of sum |L||L| of the FP32 rebuild of the whole block, the second
    hi copy equals the first and the padding columns are zero."""
    from fricc_gb300.cholesky import VvvvRebuild, _kp
    g = torch.Generator(device="cuda")
    g.manual_seed(v)
    nmo, naux = o + v, 3 * (o + v)
    A = torch.randn(naux, nmo, nmo, generator=g, device="cuda", dtype=torch.float64) * 0.05
    Lf = torch.triu(A) + torch.triu(A, 1).transpose(1, 2)
    R = VvvvRebuild(Lf, o)
    vv = v * v
    out = torch.full((vv, _kp(vv)), float("nan"), dtype=torch.bfloat16, device="cuda")
    Bt = R.rebuild_split_b(out)
    W = R.rebuild()
    R.check()
    torch.cuda.synchronize()
    assert not bool(torch.isnan(Bt).any())
    assert torch.equal(Bt[:, :vv], Bt[:, 2 * vv:3 * vv]) and bool((Bt[:, 3 * vv:] == 0).all())
    B4 = Bt[:, :vv].reshape(v, v, v, v)  # [a, b, c, d]
    assert torch.equal(B4, B4.permute(1, 0, 3, 2))
    L4 = Bt[:, vv:2 * vv].reshape(v, v, v, v)
    assert torch.equal(L4, L4.permute(1, 0, 3, 2))
    hi, lo = Bt[:, :vv].double(), Bt[:, vv:2 * vv].double()
    ref = W[:, :vv].double().T  # W[(c,d), (a,b)] = (ac|bd) -> [q=(a,b)][k=(c,d)]
    Lv = Lf[:, o:, o:].abs()
    scale = torch.einsum("Pac,Pbd->abcd", Lv, Lv).reshape(vv, vv)
    assert float(((hi + lo - ref).abs() / scale).max()) < 2.0 ** -14


@pytest.mark.parametrize("sums", ["dense", "fp32", "pairs"])
def test_split_iteration_delta_e_sums(gpulib, systems, sums):
    from fricc_gb300.friccsd import FRICCSDGPU
    s, E, Es = systems
    t1, t2 = [torch.from_numpy(x).cuda() for x in s.mp2_amplitudes()]
    fp = FRICCSDGPU(E, {"m_keep": 20000}, precision="fp64")
    sp = FRICCSDGPU(Es, {"m_keep": 20000}, precision="split", split_sparse=sums)
    for it in range(3):
        rn = [0.3 + 0.1 * it, 0.4]
        a1, a2 = fp.update_amps(t1, t2, rn=rn)
        sp.update_amps(t1, t2, rn=rn)
        assert abs(fp.read_energy()[0] - sp.read_energy()[0]) < 1e-6
        t1, t2 = a1, a2


def test_split_iteration_delta_e(gpulib, systems):
    from fricc_gb300.friccsd import FRICCSDGPU
    s, E, Es = systems
    t1, t2 = [torch.from_numpy(x).cuda() for x in s.mp2_amplitudes()]
    m = 20000
    fp = FRICCSDGPU(E, {"m_keep": m}, precision="fp64")
    sp = FRICCSDGPU(Es, {"m_keep": m}, precision="split")
    a1, a2 = t1, t2
    b1, b2 = t1, t2
    worst = 0.0
    for it in range(6):
        rn = [0.1 + 0.13 * it, 0.77 - 0.09 * it]
        a1, a2 = fp.update_amps(a1, a2, rn=rn)
        b1, b2 = sp.update_amps(b1, b2, rn=rn)
        ea, eb = fp.read_energy()[0], sp.read_energy()[0]
        worst = max(worst, abs(ea - eb))
    assert worst < 1e-6, worst
    assert Es.vvvv_rebuild.rebuilds >= 6


def test_split_rebuild_once_same_as_every_iteration(gpulib, systems):
    from fricc_gb300.friccsd import FRICCSDGPU
    s, E, Es = systems
    t1, t2 = [torch.from_numpy(x).cuda() for x in s.mp2_amplitudes()]
    a = FRICCSDGPU(Es, {"m_keep": 20000}, precision="split")
    b = FRICCSDGPU(Es, {"m_keep": 20000}, precision="split", rebuild_vvvv=False)
    for it in range(3):
        rn = [0.2 + 0.1 * it, 0.6]
        a1, a2 = a.update_amps(t1, t2, rn=rn)
        b1, b2 = b.update_amps(t1, t2, rn=rn)
        assert torch.equal(a2, b2) and torch.equal(a1, b1)  # the rebuild is deterministic
        t1, t2 = a1, a2


def test_split_graph_replay_matches_eager(gpulib, systems):
    from fricc_gb300.friccsd import FRICCSDGPU
    s, E, Es = systems
    t1, t2 = [torch.from_numpy(x).cuda() for x in s.mp2_amplitudes()]
    g = FRICCSDGPU(Es, {"m_keep": 20000}, precision="split", graph=True)
    e = FRICCSDGPU(Es, {"m_keep": 20000}, precision="split")
    a1, a2, b1, b2 = t1, t2, t1, t2
    for it in range(4):
        rn = [0.15 + 0.2 * it, 0.5]
        a1, a2 = g.update_amps(a1, a2, rn=rn)
        b1, b2 = e.update_amps(b1, b2, rn=rn)
        assert abs(g.read_energy()[0] - e.read_energy()[0]) < 1e-14
    torch.testing.assert_close(a2, b2, rtol=1e-13, atol=1e-18)


def test_split_requires_split_eris(gpulib, systems):
    from fricc_gb300.friccsd import FRICCSDGPU
    s, E, Es = systems
    with pytest.raises(ValueError):
        FRICCSDGPU(E, {"m_keep": 100}, precision="split")
    with pytest.raises(ValueError):
        FRICCSDGPU(Es, {"m_keep": 100}, precision="df64")


def test_device_system_recipe(gpulib):
    """DeviceSystem draws the synthetic recipe on the GPU: sorted orbital
    energies in their ranges, L symmetric with the normalised spread,
    reproducible per seed, and integral blocks the solvers accept."""
    from fricc_gb300.cholesky import split_eris
    from fricc_gb300.rccsd_dense import DeviceERIs
    from fricc_gb300.synthetic import DeviceSystem
    a = DeviceSystem(6, 30, 288, 0.05, seed=7)
    b = DeviceSystem(6, 30, 288, 0.05, seed=7)
    assert torch.equal(a.L, b.L) and torch.equal(a.mo_energy, b.mo_energy)
    e = a.mo_energy
    assert bool((e[:6] >= -1.5).all() and (e[:6] <= -0.3).all() and (e[6:] >= 0.2).all() and (e[6:] <= 3.0).all())
    assert bool((e[:6].diff() >= 0).all() and (e[6:].diff() >= 0).all())
    assert torch.equal(a.L, a.L.transpose(1, 2))
    assert abs(float(a.L.std()) * 288 ** 0.5 / 0.05 - 1.0) < 0.05
    E = DeviceERIs.from_system(a)
    Es = split_eris(a)
    La = a.L[:, :6, 6:].abs().reshape(288, -1)
    scale = (La.T @ La).reshape(6, 30, 6, 30)
    assert float(((Es.ovov - E.ovov).abs() / scale).max()) < 1e-11


def test_split_kernel_loop(gpulib, systems):
    """FRICCSDGPU.kernel (the reference's loop) in the split form, against
    the FP64 form's loop with the same draws."""
    from fricc_gb300.batch import mp2_device
    from fricc_gb300.friccsd import FRICCSDGPU
    from fricc_gb300.rng import GlibcRand
    s, E, Es = systems
    runs = []
    for eris, prec in ((Es, "split"), (E, "fp64")):
        cc = FRICCSDGPU(eris, {"m_keep": 20000}, rn_draw=GlibcRand(77), precision=prec)
        conv, e, t1, t2, energies = cc.kernel(*mp2_device(eris), max_cycle=6)
        runs.append(np.array(energies))
    assert len(runs[0]) == len(runs[1]) or abs(len(runs[0]) - len(runs[1])) <= 1
    n = min(len(runs[0]), len(runs[1]))
    assert np.max(np.abs(runs[0][:n] - runs[1][:n])) < 1e-6


@pytest.mark.parametrize("o,v", [(5, 21), (7, 33)])
def test_split_odd_sizes(gpulib, o, v):
    """Odd nocc and nvir (odd row lengths everywhere, partial tiles, the
    FP32 fallback's padded rows) in the split form, against FP64."""
    from fricc_gb300.batch import mp2_device
    from fricc_gb300.cholesky import split_eris
    from fricc_gb300.friccsd import FRICCSDGPU
    from fricc_gb300.rccsd_dense import DeviceERIs
    from fricc_gb300.synthetic import SyntheticSystem
    s = SyntheticSystem(o, v, 6 * (o + v), 0.05, 11)
    E, Es = DeviceERIs.from_system(s), split_eris(s)
    m = (o * o * v * v) // 8
    fp = FRICCSDGPU(E, {"m_keep": m}, precision="fp64")
    sp = FRICCSDGPU(Es, {"m_keep": m}, precision="split")
    t1, t2 = mp2_device(E)
    for it in range(3):
        rn = [0.11 + 0.2 * it, 0.7]
        a1, a2 = fp.update_amps(t1, t2, rn=rn)
        sp.update_amps(t1, t2, rn=rn)
        assert abs(fp.read_energy()[0] - sp.read_energy()[0]) < 1e-6
        t1, t2 = a1, a2
