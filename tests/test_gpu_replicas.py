"""The fused replica batch: R replicas of one system, each kernel launched
once for all of them (fricc_gb300.replicas.FusedReplicaBatch).

* Each replica's trajectory -- E_corr every iteration, t1 and t2 after
  several -- is bit for bit the one a lone FRICCSDGPU solve with the same
  seed and precision gives (FP64, FP32-pair and split-BF16x3 forms; the
  replica-batched tensor-core GEMM also against gemm_tc per replica).
* Both batched compressions of every replica keep the lone solve's entries
  bit for bit (o20v100, m = 200,000, 16 replicas).
* A bounded device wait that runs out inside the batched compression is
  reported by fricc_spb_status with the failing replica; the next
  compression on the same handle keeps the oracle's entries bit for bit.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SETTINGS = {"compression": "fri", "sampling_method": "systematic", "verbose": False,
            "compressed_contractions": ["O^2V^4", "O^3V^3", "O^4V^2"]}


def _bits(t):
    return t.contiguous().view(torch.int64)


def _lone(E, m, seed, precision, steps):
    from fricc_gb300.batch import mp2_device
    from fricc_gb300.friccsd import FRICCSDGPU
    from fricc_gb300.rng import GlibcRand
    lone = FRICCSDGPU(E, dict(SETTINGS, m_keep=m), rn_draw=GlibcRand(seed), precision=precision)
    t1, t2 = mp2_device(E)
    energies = []
    for _ in range(steps):
        t1, t2 = lone.update_amps(t1, t2)
        energies.append(lone.read_energy()[0])
    return lone, t1, t2, energies


@pytest.mark.parametrize("precision", ["fp64", "df64"])
def test_fused_replicas_equal_their_lone_solves(gpulib, precision):
    from fricc_gb300.rccsd_dense import DeviceERIs
    from fricc_gb300.replicas import FusedReplicaBatch
    from fricc_gb300.synthetic import SyntheticSystem
    E = DeviceERIs.from_system(SyntheticSystem(6, 24, 120, 0.05, 3))
    m, seeds, steps = 3000, [7, 11, 12345], 3
    fb = FusedReplicaBatch(E, {"m_keep": m}, seeds, precision=precision)
    for _ in range(steps):
        fb.step()
    for r, seed in enumerate(seeds):
        _, t1, t2, energies = _lone(E, m, seed, precision, steps)
        assert energies == fb.history[r], (r, energies, fb.history[r])
        assert torch.equal(_bits(t1), _bits(fb.t1[r])), r
        assert torch.equal(_bits(t2), _bits(fb.t2[r])), r
    assert len({h[-1] for h in fb.history}) == len(seeds)   # distinct seeds, distinct trajectories


def test_fused_o20v100_sixteen_replicas_compress_and_step_as_alone(gpulib):
    from fricc_gb300 import _lib as L
    from fricc_gb300.rccsd_dense import DeviceERIs
    from fricc_gb300.replicas import FusedReplicaBatch
    from fricc_gb300.synthetic import WORKLOADS, make_system
    w = WORKLOADS["o20v100x64"]
    m = w["m"]
    E = DeviceERIs.from_system(make_system("o20v100x64", seed=0))
    seeds = list(range(100, 116))
    fb = FusedReplicaBatch(E, {"m_keep": m}, seeds, precision="fp64")
    fb.step()
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for r in (0, 7, 15):
        lone, t1, t2, energies = _lone(E, m, seeds[r], "fp64", 1)
        assert energies == fb.history[r]
        assert torch.equal(_bits(t2), _bits(fb.t2[r])), r
        for which, h in ((0, lone._sp), (1, lone._sp_w)):
            flat = np.empty(m, dtype=np.int64)
            vals = np.empty(m, dtype=np.float64)
            L.check(gpulib.fricc_sp_export(h.h, ctypes.c_void_p(flat.ctypes.data), ctypes.c_void_p(vals.ctypes.data),
                                           st))
            bf, bv = fb.export(which, r)
            assert np.array_equal(flat, bf) and np.array_equal(vals.view(np.int64), bv.view(np.int64)), (r, which)
    mean, var = fb.stats()
    assert np.isfinite(mean) and var > 0.0


def test_batched_compression_wait_runs_out_and_recovers(gpulib, oracle):
    from fricc_gb300 import _lib as L
    rng = np.random.default_rng(21)
    R, dims, m = 2, (8, 8, 40, 40), 20000
    x_h = rng.standard_normal((R,) + dims) * rng.random((R,) + dims) ** 4
    x = torch.from_numpy(x_h).cuda()
    draws = [[0.5, 0.25], [0.125, 0.875]]
    rn = torch.tensor(draws, dtype=torch.float64).cuda()
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    spb = ctypes.c_void_p()
    L.check(gpulib.fricc_spb_create(R, L.i64arr(dims), m, st, ctypes.byref(spb)))
    try:
        rep = ctypes.c_int(-2)
        L.check(gpulib.fricc_tune_set(3, 2000))   # knob 3: the test-only wait of 2000 polls
        try:
            L.check(gpulib.fricc_spb_recompress_pair(spb, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(rn.data_ptr()),
                                                     st))
            assert gpulib.fricc_spb_status(spb, ctypes.byref(rep)) == 5   # FRICC_ERR_TIMEOUT
            assert rep.value in range(R)
        finally:
            L.check(gpulib.fricc_tune_set(3, -1))
        # the same handle, re-compressed: every replica's entries as the oracle's
        L.check(gpulib.fricc_spb_recompress_pair(spb, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(rn.data_ptr()), st))
        L.check(gpulib.fricc_spb_status(spb, ctypes.byref(rep)))
        assert rep.value == -1
        for r in range(R):
            for which in (0, 1):
                flat = np.empty(m, dtype=np.int64)
                vals = np.empty(m, dtype=np.float64)
                L.check(gpulib.fricc_spb_export(spb, which, r, ctypes.c_void_p(flat.ctypes.data),
                                                ctypes.c_void_p(vals.ctypes.data), st))
                ref = oracle.SparseTensor4d(x_h[r], dims, m, "fri", "systematic", rn=draws[r][which])
                assert np.array_equal(flat, ref.flat), (r, which)
                assert np.array_equal(vals.view(np.int64), ref.vals.view(np.int64)), (r, which)
    finally:
        gpulib.fricc_spb_destroy(spb)


@pytest.mark.parametrize("case", ["shared_a", "batched_a", "swap", "split_k", "pair_fallback"])
def test_gemm_tc_rep_equals_gemm_tc_per_replica(gpulib, case):
    """The replica-batched tensor-core GEMM against gemm_tc called replica by
    replica: bit for bit, through each of its routes (a constant split A,
    batch-flattened rows, the narrow-side swap, split K with per-replica
    partials, and the FP32-pair fallback)."""
    from fricc_gb300.cholesky import gemm_tc, gemm_tc_rep, split_a
    g = torch.Generator(device="cuda").manual_seed(3)
    R = 3

    def rnd(*shape):
        return torch.randn(*shape, generator=g, device="cuda", dtype=torch.float64)
    a_split = None
    if case == "shared_a":        # R = ovvv . t1^T: a constant A, per-replica B (a transposed view)
        A, B, C0 = rnd(8000, 100), rnd(R, 20, 100).transpose(1, 2), rnd(R, 8000, 20)
        a_split = split_a(A)
        lone = lambda r, C: gemm_tc(A, B[r], C, -1.0, 1.0, a_split=a_split)  # noqa: E731
        alpha, beta = -1.0, 1.0
    elif case == "batched_a":     # the X t1 term: a batched A, B one per replica (batch stride 0)
        A = rnd(R, 100, 20, 100).transpose(2, 3)
        B = rnd(R, 1, 20, 100).expand(R, 100, 20, 100)
        C0 = rnd(R, 100, 100, 100)
        lone = lambda r, C: gemm_tc(A[r], B[r], C, -1.0, 1.0)  # noqa: E731
        alpha, beta = -1.0, 1.0
    elif case == "swap":          # Loo t2: M = 20 <= 64 < N
        A, B, C0 = rnd(R, 20, 20).transpose(1, 2), rnd(R, 20, 40000), rnd(R, 20, 40000)
        lone = lambda r, C: gemm_tc(A[r], B[r], C, 1.0, 0.0)  # noqa: E731
        alpha, beta = 1.0, 0.0
    elif case == "split_k":       # cc_Foo: one 20 x 20 tile, K = 20,000
        A, B, C0 = rnd(20, 20000), rnd(R, 20, 20000).transpose(1, 2), rnd(R, 20, 20)
        a_split = split_a(A)
        lone = lambda r, C: gemm_tc(A, B[r], C, 1.0, 1.0, a_split=a_split)  # noqa: E731
        alpha, beta = 1.0, 1.0
    else:                         # few tiles, short K: the FP32-pair GEMM
        A, B, C0 = rnd(R, 20, 30), rnd(30, 20), rnd(R, 20, 20)
        lone = lambda r, C: gemm_tc(A[r], B, C, 1.0, 0.0)  # noqa: E731
        alpha, beta = 1.0, 0.0
    want = C0.clone()
    for r in range(R):
        lone(r, want[r])
    got = C0.clone()
    gemm_tc_rep(A, B, got, alpha, beta, R, a_split=a_split)
    torch.cuda.synchronize()
    assert torch.equal(_bits(got), _bits(want))
    assert not torch.equal(got, C0)


def test_fused_split_replicas_equal_their_lone_solves(gpulib):
    from fricc_gb300.cholesky import split_eris
    from fricc_gb300.replicas import FusedReplicaBatch
    from fricc_gb300.synthetic import SyntheticSystem
    E = split_eris(SyntheticSystem(10, 80, 400, 0.05, 3))
    m, seeds, steps = 32000, [7, 11, 12345], 2
    fb = FusedReplicaBatch(E, {"m_keep": m}, seeds, precision="split")
    for _ in range(steps):
        fb.step()
    for r, seed in enumerate(seeds):
        _, t1, t2, energies = _lone(E, m, seed, "split", steps)
        assert energies == fb.history[r], (r, energies, fb.history[r])
        assert torch.equal(_bits(t1), _bits(fb.t1[r])), r
        assert torch.equal(_bits(t2), _bits(fb.t2[r])), r


def test_fused_split_declines_terms_too_small_for_the_tensor_cores(gpulib):
    from fricc_gb300.cholesky import split_eris
    from fricc_gb300.replicas import FusedReplicaBatch
    from fricc_gb300.synthetic import SyntheticSystem
    E = split_eris(SyntheticSystem(6, 24, 120, 0.05, 3))
    with pytest.raises(ValueError):
        FusedReplicaBatch(E, {"m_keep": 3000}, [1, 2], precision="split")


@pytest.mark.parametrize("precision", ["df64", "split"])
def test_fused_replicas_graph_replays_equal_eager(gpulib, precision):
    """graph=True: the first batch step eager, the second captured into one
    CUDA graph and every later step a replay of it; each replica's E_corr at
    every step and t1, t2 after four steps are bit for bit the eager batch's."""
    from fricc_gb300.replicas import FusedReplicaBatch
    from fricc_gb300.synthetic import SyntheticSystem
    if precision == "split":
        from fricc_gb300.cholesky import split_eris
        E, m = split_eris(SyntheticSystem(10, 80, 400, 0.05, 3)), 32000
    else:
        from fricc_gb300.rccsd_dense import DeviceERIs
        E, m = DeviceERIs.from_system(SyntheticSystem(6, 24, 120, 0.05, 3)), 3000
    seeds, steps = [7, 11, 12345], 4
    eager = FusedReplicaBatch(E, {"m_keep": m}, seeds, precision=precision)
    graph = FusedReplicaBatch(E, {"m_keep": m}, seeds, precision=precision, graph=True)
    for _ in range(steps):
        eager.step()
        graph.step()
    assert graph._g is not None
    assert graph.history == eager.history
    assert torch.equal(_bits(graph.t1), _bits(eager.t1)) and torch.equal(_bits(graph.t2), _bits(eager.t2))
