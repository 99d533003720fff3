"""Index bookkeeping of the einsum-to-GEMM mapping, on the CPU.

The FP32-pair GEMM itself needs a GPU; here it is replaced by an FP64
matmul honouring the same (A, B, C, alpha, beta) contract, so the test
checks only how einsum_df groups, permutes and reshapes the operands."""
import pytest
import torch

from fricc_gb300 import rccsd_dense as D


@pytest.fixture
def cpu_gemm(monkeypatch):
    def fake(A, B, C, alpha=1.0, beta=0.0):
        R = torch.matmul(A, B)
        C.mul_(beta).add_(R, alpha=alpha) if beta != 0.0 else C.copy_(alpha * R)
        return C
    monkeypatch.setattr(D, "gemm_df", fake)


SPECS = [
    ("kibc,jc->kibj", (3, 4, 5, 5), (4, 5)),
    ("ka,kibj->ijab", (3, 5), (3, 4, 5, 4)),
    ("kcai,jc->akij", (3, 5, 5, 4), (4, 5)),
    ("akij,kb->ijab", (5, 3, 4, 4), (3, 5)),
    ("lcki,klac->ia", (3, 5, 3, 4), (3, 3, 5, 5)),
    ("klij,ka->lija", (3, 3, 4, 4), (3, 5)),
    ("ldkc,id->lkci", (3, 5, 3, 5), (4, 5)),
    ("pr,qs->pqrs", (3, 4), (2, 5)),                 # outer product (K = 1)
    ("bij,bjk->bik", (2, 3, 4), (2, 4, 5)),          # shared batch index
    ("kcld,kd->lc", (3, 4, 2, 5), (3, 5)),           # lone-free two-index contraction
    ("abx,bc->ac", (3, 4, 2), (4, 5)),               # x summed out of A first
]


@pytest.mark.parametrize("spec,sa,sb", SPECS)
def test_einsum_df_layout(cpu_gemm, spec, sa, sb):
    g = torch.Generator().manual_seed(7)
    A = torch.randn(*sa, dtype=torch.float64, generator=g)
    B = torch.randn(*sb, dtype=torch.float64, generator=g)
    want = torch.einsum(spec, A, B)
    got = D.einsum_df(spec, A, B)
    assert got.shape == want.shape
    torch.testing.assert_close(got, want, rtol=1e-13, atol=1e-13)


def test_einsum_df_noncontiguous_operands(cpu_gemm):
    g = torch.Generator().manual_seed(3)
    A = torch.randn(5, 4, 3, 6, dtype=torch.float64, generator=g).permute(2, 0, 3, 1)   # [3,5,6,4]
    B = torch.randn(6, 4, dtype=torch.float64, generator=g)[::2]                     # [3,4] strided
    assert not A.is_contiguous() and not B.is_contiguous()
    torch.testing.assert_close(D.einsum_df("kcai,ji->kcaj", A, B), torch.einsum("kcai,ji->kcaj", A, B),
                               rtol=1e-13, atol=1e-13)


def test_einsum_df_rejects_repeated_index():
    with pytest.raises(ValueError):
        D.einsum_df("iij,jk->ik", torch.zeros(2, 2, 3, dtype=torch.float64), torch.zeros(3, 4, dtype=torch.float64))
