"""Split-precision integral rebuilds from a Cholesky factor on the tcgen05
tensor cores.

The synthetic systems define every integral block through a factor L
(``(pq|rs) = sum_P L[P,p,q] L[P,r,s]``, L symmetric in p, q).  In the
split-precision form the factor is held as BF16 hi + lo pairs and a block is
rebuilt as one BF16 GEMM over K-concatenated operands
(A' = [hi | hi | lo], B' = [hi | lo | hi]: hi.hi + hi.lo + lo.hi, FP32
accumulation in tensor memory), ~2^-16 of sum |L||L| per element.  The
(vv|vv) block is written straight into the FP32 layout of the O^2V^4
contraction (rows (c,d), columns (a,b)), so it never exists in FP64.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib as L


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _st(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _check_operand(x, name):
    if x.dtype != torch.bfloat16 or x.dim() != 2 or x.stride(1) != 1 or not x.is_cuda:
        raise ValueError(f"{name}: a CUDA bfloat16 matrix with unit column stride")
    if x.stride(0) % 8 or x.data_ptr() % 16:
        raise ValueError(f"{name}: row stride must be a multiple of 8 elements and the base 16-byte aligned")


def gemm_bf16_tn(A: torch.Tensor, B: torch.Tensor, out: torch.Tensor | None = None, f64: bool = False):
    """A [M,K] . B [N,K]^T on the tensor cores (BF16 in, FP32 accumulation);
    FP32 result, or FP64 (the FP32 sums widened exactly) with ``f64``."""
    _check_operand(A, "A")
    _check_operand(B, "B")
    M, K = A.shape
    N, K2 = B.shape
    if K2 != K:
        raise ValueError("A and B must have the same K")
    dt = torch.float64 if f64 else torch.float32
    if out is None:
        out = torch.empty(M, N, dtype=dt, device=A.device)
    if out.dtype != dt or out.dim() != 2 or out.stride(1) != 1 or out.shape != (M, N):
        raise ValueError("out: an (M, N) matrix of the result type with unit column stride")
    lib = L.load()
    fn = lib.fricc_gemm_bf16_tn_f64 if f64 else lib.fricc_gemm_bf16_tn
    L.check(fn(_p(A), A.stride(0), _p(B), B.stride(0), M, N, K, _p(out), out.stride(0), _st()))
    return out


def split_bf16x3(x: torch.Tensor, kp: int | None = None):
    """x [rows, k] FP64 -> (A', B') [rows, kp] BF16 with A' = [hi|hi|lo],
    B' = [hi|lo|hi] (kp >= 3k, a multiple of 8; padding zero)."""
    if x.dtype != torch.float64 or x.dim() != 2 or x.stride(1) != 1 or not x.is_cuda:
        raise ValueError("x: a CUDA float64 matrix with unit column stride")
    rows, k = x.shape
    kp = kp if kp is not None else -(-3 * k // 8) * 8
    if kp < 3 * k or kp % 8:
        raise ValueError("kp must be >= 3k and a multiple of 8")
    Ap = torch.empty(rows, kp, dtype=torch.bfloat16, device=x.device)
    Bp = torch.empty_like(Ap)
    L.check(L.load().fricc_split_bf16x3(_p(x), rows, k, x.stride(0), kp, _p(Ap), _p(Bp), _st()))
    return Ap, Bp


def lvv_t(Lf: torch.Tensor, nocc: int) -> torch.Tensor:
    """L_vv^T [v*v, naux] (row c*v + a = L[:, a, c]) of a factor L [naux, nmo, nmo]."""
    naux = Lf.shape[0]
    return Lf[:, nocc:, nocc:].reshape(naux, -1).t().contiguous()


class VvvvRebuild:
    """The (vv|vv) block rebuilt from the split factor: W[(c,d), (a,b)] =
    (ac|bd) in FP32 (rows of ``ldw`` = v*v floats), on demand."""

    def __init__(self, Lf: torch.Tensor, nocc: int):
        nmo = Lf.shape[1]
        self.v = nmo - nocc
        self.Ap, self.Bp = split_bf16x3(lvv_t(Lf, nocc))
        self.kp = self.Ap.shape[1]
        self.ldw = self.v * self.v
        self.W = None

    def rebuild(self, out: torch.Tensor | None = None) -> torch.Tensor:
        v = self.v
        if out is None:
            if self.W is None:
                self.W = torch.empty(v * v, self.ldw, dtype=torch.float32, device=self.Ap.device)
            out = self.W
        L.check(L.load().fricc_vvvv_rebuild_bf16x3(_p(self.Ap), _p(self.Bp), v, self.kp, _p(out), self.ldw, _st()))
        return out
