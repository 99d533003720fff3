"""The library's GEMMs -- FP32 pairs (fricc_gemm_df) and FP64 DFMA
(fricc_gemm_f64) -- against torch FP64 on the shapes the iteration uses:
long-K (split) reductions, transposed and strided operands, batches with a
shared operand, alpha/beta accumulation."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
GEMMS = ["gemm_df", "gemm_f64"]


def _gemm(name):
    from fricc_gb300 import rccsd_dense
    return getattr(rccsd_dense, name)


def _rel(a, b, scale):
    return float((a - b).abs().max() / scale)


@pytest.mark.parametrize("M,N,K", [(30, 150, 675000), (30, 30, 675000), (150, 150, 135000), (4500, 30, 150),
                                   (30, 40000, 30), (65, 67, 129), (1, 1, 1), (7, 9, 33), (129, 31, 17),
                                   (33, 161, 5), (2, 3, 100000), (1, 4500, 4500), (3, 22500, 4500),
                                   (4500, 1, 4500), (900, 4, 77)])
@pytest.mark.parametrize("name", GEMMS)
def test_gemm_2d(gpulib, name, M, N, K):
    gemm_df = _gemm(name)
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N)
    A = torch.randn(M, K, dtype=torch.float64, device="cuda", generator=g)
    B = torch.randn(N, K, dtype=torch.float64, device="cuda", generator=g).T   # transposed operand
    C0 = torch.randn(M, N, dtype=torch.float64, device="cuda", generator=g)
    C = C0.clone()
    gemm_df(A, B, C, alpha=-0.5, beta=1.0)
    ref = C0 - 0.5 * (A @ B)
    scale = float((A.abs() @ B.abs()).max()) * 0.5 + float(C0.abs().max())
    assert _rel(C, ref, scale) < 1e-13


@pytest.mark.parametrize("name", GEMMS)
def test_gemm_batched_shared_and_deterministic(gpulib, name):
    gemm_df = _gemm(name)
    g = torch.Generator(device="cuda").manual_seed(5)
    b, v, o = 64, 40, 7
    L = torch.randn(v, v, dtype=torch.float64, device="cuda", generator=g)
    T = torch.randn(b, v, v, dtype=torch.float64, device="cuda", generator=g)
    C = torch.empty(b, v, v, dtype=torch.float64, device="cuda")
    gemm_df(L.unsqueeze(0).expand(b, v, v), T, C)
    assert _rel(C, L @ T, float((L.abs() @ T.abs()).max())) < 1e-13
    X = torch.randn(b, 2, o, v, dtype=torch.float64, device="cuda", generator=g)
    t1 = torch.randn(o, v, dtype=torch.float64, device="cuda", generator=g)
    D = torch.zeros(b, v, v, dtype=torch.float64, device="cuda")
    gemm_df(X[:, 0].transpose(1, 2), t1.unsqueeze(0).expand(b, o, v), D, -1.0, 1.0)
    ref = -(X[:, 0].transpose(1, 2) @ t1)
    assert _rel(D, ref, float((X.abs()[:, 0].transpose(1, 2) @ t1.abs()).max())) < 1e-13
    D2 = torch.zeros_like(D)
    gemm_df(X[:, 0].transpose(1, 2), t1.unsqueeze(0).expand(b, o, v), D2, -1.0, 1.0)
    assert torch.equal(D, D2)


@pytest.mark.parametrize("name", GEMMS)
def test_gemm_row_major_b(gpulib, name):
    """B with unit stride along N (the staging path for n-contiguous B)."""
    gemm_df = _gemm(name)
    g = torch.Generator(device="cuda").manual_seed(11)
    for (M, N, K) in ((45, 151, 300), (300, 30, 4500), (31, 33, 1000)):
        A = torch.randn(K, M, dtype=torch.float64, device="cuda", generator=g).T   # m-contiguous A
        B = torch.randn(K, N, dtype=torch.float64, device="cuda", generator=g)
        C = torch.empty(M, N, dtype=torch.float64, device="cuda")
        gemm_df(A, B, C)
        assert _rel(C, A @ B, float((A.abs() @ B.abs()).max())) < 1e-13


@pytest.mark.parametrize("spec,sa,sb", [("kibc,jc->kibj", (30, 30, 150, 150), (30, 150)),
                                        ("ka,kibj->ijab", (30, 150), (30, 30, 150, 30)),
                                        ("lcki,klac->ia", (30, 150, 30, 30), (30, 30, 150, 150)),
                                        ("lkci,la->akic", (30, 30, 150, 30), (30, 150))])
@pytest.mark.parametrize("name", GEMMS)
def test_einsum_df_matches_einsum(gpulib, spec, sa, sb, name):
    """The iteration's two-operand einsums on the library's GEMMs against FP64 einsum."""
    from fricc_gb300.rccsd_dense import einsum_df
    g = torch.Generator(device="cuda").manual_seed(len(spec))
    A = torch.randn(*sa, dtype=torch.float64, device="cuda", generator=g)
    B = torch.randn(*sb, dtype=torch.float64, device="cuda", generator=g)
    ref = torch.einsum(spec, A, B)
    got = einsum_df(spec, A, B, gemm=_gemm(name))
    assert got.shape == ref.shape
    assert _rel(got, ref, float(torch.einsum(spec, A.abs(), B.abs()).max())) < 1e-13


def test_gemm_f64_deterministic_split_k_and_zero_k(gpulib):
    """Split-K partials are summed in slice order: repeated calls agree bit
    for bit; K = 0 leaves beta C."""
    from fricc_gb300.rccsd_dense import gemm_f64
    g = torch.Generator(device="cuda").manual_seed(3)
    A = torch.randn(30, 675000, dtype=torch.float64, device="cuda", generator=g)
    B = torch.randn(675000, 150, dtype=torch.float64, device="cuda", generator=g)
    C1 = torch.empty(30, 150, dtype=torch.float64, device="cuda")
    C2 = torch.empty_like(C1)
    gemm_f64(A, B, C1)
    gemm_f64(A, B, C2)
    assert torch.equal(C1, C2)
    C0 = torch.randn(5, 7, dtype=torch.float64, device="cuda", generator=g)
    C = C0.clone()
    gemm_f64(torch.empty(5, 0, dtype=torch.float64, device="cuda"),
             torch.empty(0, 7, dtype=torch.float64, device="cuda"), C, 1.0, 2.0)
    assert torch.equal(C, 2.0 * C0)


@pytest.mark.parametrize("M,N,K,bt", [(1, 4500, 4500, 1), (1, 150, 4500, 30), (4500, 1, 4500, 1), (4, 2, 9, 7)])
def test_gemm_f64_skinny_strided(gpulib, M, N, K, bt):
    """The dot-product paths of fricc_gemm_f64 (a few rows or columns) with
    strided, batched and shared operands, alpha/beta."""
    from fricc_gb300.rccsd_dense import gemm_f64
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    A = torch.randn(bt, K, M, dtype=torch.float64, device="cuda", generator=g).transpose(1, 2)  # m-contiguous
    B = torch.randn(K, N, dtype=torch.float64, device="cuda", generator=g).unsqueeze(0).expand(bt, K, N)
    C0 = torch.randn(bt, M, N, dtype=torch.float64, device="cuda", generator=g)
    C = C0.clone()
    gemm_f64(A if bt > 1 else A[0], B if bt > 1 else B[0], C if bt > 1 else C[0], 0.75, -1.0)
    ref = 0.75 * (A @ B) - C0
    scale = float((A.abs() @ B.abs()).max()) + float(C0.abs().max())
    assert _rel(C, ref, scale) < 1e-13
