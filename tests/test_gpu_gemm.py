"""The FP32-pair GEMM (fricc_gemm_df) against cuBLAS FP64 on the shapes the
iteration uses: long-K (split) reductions, transposed and strided operands,
batches with a shared operand, alpha/beta accumulation."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _rel(a, b, scale):
    return float((a - b).abs().max() / scale)


@pytest.mark.parametrize("M,N,K", [(30, 150, 675000), (30, 30, 675000), (150, 150, 135000), (4500, 30, 150),
                                   (30, 40000, 30), (65, 67, 129), (1, 1, 1), (7, 9, 33), (129, 31, 17),
                                   (33, 161, 5), (2, 3, 100000)])
def test_gemm_df_2d(gpulib, M, N, K):
    from fricc_gb300.rccsd_dense import gemm_df
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N)
    A = torch.randn(M, K, dtype=torch.float64, device="cuda", generator=g)
    B = torch.randn(N, K, dtype=torch.float64, device="cuda", generator=g).T   # transposed operand
    C0 = torch.randn(M, N, dtype=torch.float64, device="cuda", generator=g)
    C = C0.clone()
    gemm_df(A, B, C, alpha=-0.5, beta=1.0)
    ref = C0 - 0.5 * (A @ B)
    scale = float((A.abs() @ B.abs()).max()) * 0.5 + float(C0.abs().max())
    assert _rel(C, ref, scale) < 1e-13


def test_gemm_df_batched_shared_and_deterministic(gpulib):
    from fricc_gb300.rccsd_dense import gemm_df
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


def test_gemm_df_row_major_b(gpulib):
    """B with unit stride along N (the staging path for n-contiguous B)."""
    from fricc_gb300.rccsd_dense import gemm_df
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
def test_einsum_df_matches_einsum(gpulib, spec, sa, sb):
    """The iteration's two-operand einsums on the float-pair GEMM against FP64 einsum."""
    from fricc_gb300.rccsd_dense import einsum_df
    g = torch.Generator(device="cuda").manual_seed(len(spec))
    A = torch.randn(*sa, dtype=torch.float64, device="cuda", generator=g)
    B = torch.randn(*sb, dtype=torch.float64, device="cuda", generator=g)
    ref = torch.einsum(spec, A, B)
    got = einsum_df(spec, A, B)
    assert got.shape == ref.shape
    assert _rel(got, ref, float(torch.einsum(spec, A.abs(), B.abs()).max())) < 1e-13
