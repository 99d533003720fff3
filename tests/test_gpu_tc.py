"""The tcgen05 BF16 GEMM and the split-BF16x3 rebuilds (fricc_gb300/csrc/gemm_tc.cu).

* integer-valued BF16 operands make every FP32 sum exact, so the tensor-core
  result must equal the FP64 product bit for bit: this pins the operand
  layouts (TMA boxes, 128-byte swizzle, MMA descriptors), the K tail, the M
  and N edge tiles and the tile order;
* random operands: within FP32 accumulation error of the FP64 product;
* split-BF16x3 products and the (vv|vv) rebuild: within 2^-14 of
  sum |x||y| of the FP64 product (the BF16 hi + lo pair keeps ~16 bits).
"""
import pytest
import torch

pytestmark = pytest.mark.gpu


def _ints(shape, lo, hi, seed):
    g = torch.Generator().manual_seed(seed)
    return torch.randint(lo, hi + 1, shape, generator=g).to(torch.bfloat16).cuda()


@pytest.mark.parametrize("M,N,K", [(128, 256, 64), (300, 520, 200), (2100, 300, 72), (77, 19, 8), (2100, 64, 200), (300, 33, 1000)])
def test_gemm_integer_exact(gpulib, M, N, K):
    from fricc_gb300.cholesky import gemm_bf16_tn
    A = _ints((M, K), -8, 8, 1)
    B = _ints((N, K), -8, 8, 2)
    C = gemm_bf16_tn(A, B)
    ref = (A.double() @ B.double().T).float()
    assert torch.equal(C, ref)
    C64 = gemm_bf16_tn(A, B, f64=True)
    assert torch.equal(C64, A.double() @ B.double().T)


def test_gemm_strided_operands(gpulib):
    from fricc_gb300.cholesky import gemm_bf16_tn
    Abig = _ints((260, 136), -4, 4, 3)
    Bbig = _ints((140, 136), -4, 4, 4)
    A, B = Abig[:, :120], Bbig[3:, :120]  # row strides 136, K = 120
    out = torch.full((260, 140), -1.0, dtype=torch.float32, device="cuda")
    C = gemm_bf16_tn(A, B, out=out[:, :137])  # output row stride 140
    assert torch.equal(C, (A.double() @ B.double().T).float())
    assert bool((out[:, 137:] == -1.0).all())


def test_gemm_random_fp32_accuracy(gpulib):
    from fricc_gb300.cholesky import gemm_bf16_tn
    g = torch.Generator().manual_seed(5)
    A = torch.randn(520, 1000, generator=g).to(torch.bfloat16).cuda()
    B = torch.randn(390, 1000, generator=g).to(torch.bfloat16).cuda()
    C = gemm_bf16_tn(A, B, f64=True)
    ref = A.double() @ B.double().T
    scale = A.double().abs() @ B.double().abs().T
    assert bool(((C - ref).abs() <= 1e-6 * scale).all())


def test_split_bf16x3_product(gpulib):
    from fricc_gb300.cholesky import gemm_bf16_tn, split_bf16x3
    g = torch.Generator().manual_seed(6)
    x = torch.randn(300, 150, generator=g, dtype=torch.float64).cuda()
    y = torch.randn(260, 150, generator=g, dtype=torch.float64).cuda() * 1e-3
    Ax, _ = split_bf16x3(x)
    _, By = split_bf16x3(y)
    assert Ax.shape == (300, 456) and bool((Ax[:, 450:] == 0).all())
    C = gemm_bf16_tn(Ax, By, f64=True)
    ref = x @ y.T
    scale = x.abs() @ y.abs().T
    err = float(((C - ref).abs() / scale).max())
    assert err < 2.0 ** -14, err
    # the split itself: hi + lo within 2^-16 of x
    hi, lo = Ax[:, :150].double(), Ax[:, 300:450].double()
    assert float(((hi + lo - x).abs() / x.abs().clamp_min(1e-300)).max()) < 2.0 ** -15


def test_vvvv_rebuild_matches_fp64(gpulib):
    from fricc_gb300.cholesky import VvvvRebuild
    from fricc_gb300.synthetic import make_system
    s = make_system("o10v40", seed=0)
    Lf = torch.from_numpy(s.L).cuda()
    o, v = s.nocc, s.nvir
    R = VvvvRebuild(Lf, o)
    W = R.rebuild()
    Lv = Lf[:, o:, o:]
    ref = torch.einsum("Pac,Pbd->cdab", Lv, Lv).reshape(v * v, v * v)
    scale = torch.einsum("Pac,Pbd->cdab", Lv.abs(), Lv.abs()).reshape(v * v, v * v)
    err = float(((W.double() - ref).abs() / scale).max())
    assert err < 2.0 ** -14, err


def _bound_ok(C, ref, scale, tol=2.0 ** -14):
    return bool(((C - ref).abs() <= tol * scale + 1e-300).all())


@pytest.mark.parametrize("case", ["2d", "2d_transposed", "a_shared", "b_shared", "beta", "splitk", "narrow_n",
                                  "narrow_m", "fallback_small"])
def test_gemm_tc_contract(gpulib, case):
    """gemm_tc follows gemm_df's contract (strided, batched with a shared
    operand, alpha/beta) within the split-BF16x3 error."""
    from fricc_gb300.cholesky import gemm_tc
    g = torch.Generator().manual_seed(11)
    r = lambda *s: torch.randn(*s, generator=g, dtype=torch.float64).cuda()
    alpha, beta = 1.0, 0.0
    if case == "2d":
        A, B = r(3000, 70), r(70, 300)
        C = torch.empty(3000, 300, dtype=torch.float64, device="cuda")
    elif case == "2d_transposed":   # A and B as transposed views
        A = r(45, 2900).T
        B = r(310, 45).T
        C = torch.empty(2900, 310, dtype=torch.float64, device="cuda")
    elif case == "a_shared":   # Lvv t2: A (v x v) shared over o^2 batches
        A = r(60, 60).unsqueeze(0).expand(400, 60, 60)
        B = r(400, 60, 60)
        C = torch.empty(400, 60, 60, dtype=torch.float64, device="cuda")
    elif case == "b_shared":   # X t1: B shared over batches, A a transposed batched view
        A = r(400, 20, 60).transpose(1, 2)
        B = r(20, 60).unsqueeze(0).expand(400, 20, 60)
        C = torch.empty(400, 60, 60, dtype=torch.float64, device="cuda")
    elif case == "beta":
        A, B = r(6000, 40), r(40, 200)
        C = r(6000, 200)
        alpha, beta = -1.0, 1.0
    elif case == "narrow_n":   # N = nocc: 64-wide tiles (the [o v v, v] x t1^T GEMMs)
        A, B = r(30 * 150 * 150 // 10, 150), r(150, 30)
        C = torch.empty(A.shape[0], 30, dtype=torch.float64, device="cuda")
    elif case == "narrow_m":   # M = nocc: operands swapped so the narrow side is N
        A, B = r(30, 3000), r(3000, 7000)
        C = r(30, 7000)
        alpha, beta = 1.0, -1.0
    elif case == "splitk":     # one output tile, long K: split K, ordered reduction
        A, B = r(30, 20000), r(20000, 150)
        C = r(30, 150)
        alpha, beta = 0.5, 2.0
    else:                      # few tiles, short K: the FP32-pair GEMM
        A, B = r(30, 300), r(300, 150)
        C = torch.empty(30, 150, dtype=torch.float64, device="cuda")
    C0 = C.clone()
    ref = alpha * torch.matmul(A, B) + beta * C0
    scale = abs(alpha) * torch.matmul(A.abs(), B.abs()) + abs(beta) * C0.abs()
    gemm_tc(A, B, C, alpha, beta)
    assert _bound_ok(C, ref, scale)
    if case == "fallback_small":
        assert float(((C - ref).abs() / scale).max()) < 1e-12  # FP32 pairs, not BF16


def test_gemm_tc_splitk_deterministic(gpulib):
    from fricc_gb300.cholesky import gemm_tc
    g = torch.Generator().manual_seed(12)
    A = torch.randn(200, 30000, generator=g, dtype=torch.float64).cuda()
    B = torch.randn(30000, 200, generator=g, dtype=torch.float64).cuda()
    C1 = torch.empty(200, 200, dtype=torch.float64, device="cuda")
    C2 = torch.empty_like(C1)
    gemm_tc(A, B, C1)
    gemm_tc(A, B, C2)
    assert torch.equal(C1, C2)
    ref, scale = A @ B, A.abs() @ B.abs()
    assert _bound_ok(C1, ref, scale)
