"""The replica-batched contraction plumbing on the CPU: einsum_rep groups
each replica's operands as einsum_df does for one and runs the replica as a
second GEMM batch level; with a plain matmul standing in for the device
GEMM, every contraction the fused replica iteration issues matches
torch.einsum replica by replica (shared and stacked operands, fresh outputs
and alpha/beta into an existing one)."""
import pytest
import torch

from fricc_gb300.replicas import einsum_rep

O, V, R = 3, 5, 4
SPECS = [  # (spec, A stacked, B stacked): the contractions of the fused iteration
    ("lcki,klac->ia", False, True), ("kibc,jc->kibj", False, True), ("ka,kibj->ijab", True, True),
    ("kcai,jc->akij", False, True), ("akij,kb->ijab", True, True), ("lcki,jc->klij", False, True),
    ("kclj,ic->klij", False, True), ("kcld,ic->kild", False, True), ("kild,jd->klij", True, True),
    ("kcli,la->akic", False, True), ("ldkc,id->lkci", False, True), ("lkci,la->akic", True, True),
    ("lcki,la->akci", False, True), ("lckd,id->lkci", False, True), ("lkci,la->akci", True, True),
    ("klij,ka->lija", True, True), ("lija,lb->ijab", True, True),
]


def _mm(A, B, C, alpha=1.0, beta=0.0):
    C.copy_(alpha * torch.matmul(A, B) + beta * C)
    return C


def _operand(idx, stacked, g):
    shape = [O if c in "ijkl" else V for c in idx]
    return torch.randn(([R] if stacked else []) + shape, generator=g, dtype=torch.float64)


@pytest.mark.parametrize("spec,za,zb", SPECS)
def test_einsum_rep_matches_einsum_per_replica(spec, za, zb):
    g = torch.Generator().manual_seed(sum(map(ord, spec)))
    a, b = spec.split("->")[0].split(",")
    A, B = _operand(a, za, g), _operand(b, zb, g)
    got = einsum_rep(spec, A, B, _mm, za, zb, R)
    for r in range(R):
        want = torch.einsum(spec, A[r] if za else A, B[r] if zb else B)
        torch.testing.assert_close(got[r], want, rtol=1e-13, atol=1e-13)


def test_einsum_rep_accumulates_into_out():
    g = torch.Generator().manual_seed(5)
    A, B = _operand("lcki", False, g), _operand("klac", True, g)
    out = torch.randn(R, O, V, generator=g, dtype=torch.float64)
    before = out.clone()
    einsum_rep("lcki,klac->ia", A, B, _mm, False, True, R, out=out, alpha=-1.0, beta=1.0)
    for r in range(R):
        torch.testing.assert_close(out[r], before[r] - torch.einsum("lcki,klac->ia", A, B[r]), rtol=1e-13, atol=1e-13)


def test_einsum_rep_rejects_an_index_summed_over_one_operand():
    with pytest.raises(ValueError):
        einsum_rep("ijk,jl->il", torch.zeros(R, 2, 2, 2, dtype=torch.float64), torch.zeros(R, 2, 2,
                   dtype=torch.float64), _mm, True, True, R)
