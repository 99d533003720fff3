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
import threading

import torch

from . import _lib as L


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _st(stream=None):
    return ctypes.c_void_p(stream.cuda_stream) if stream is not None else L.cur_stream()


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


def _kp(k: int) -> int:
    return -(-3 * k // 8) * 8


def _split_view(x, rows, k, ri, sro, sri, sk, want_a, want_b):
    kp = _kp(k)
    Ap = torch.empty(rows, kp, dtype=torch.bfloat16, device=x.device) if want_a else None
    Bp = torch.empty(rows, kp, dtype=torch.bfloat16, device=x.device) if want_b else None
    L.check(L.load().fricc_split_bf16x3_strided(_p(x), rows, k, ri, sro, sri, sk, kp,
                                                _p(Ap) if want_a else None, _p(Bp) if want_b else None, _st()))
    return Ap if want_a else Bp


# the tensor-core path needs enough work units to spread over the SMs: a
# GEMM with few output tiles and a long K (the O^2V^3 T1 term, cc_Foo,
# cc_Fvv) splits K; one with few tiles and a short K stays on the FP32-pair
# GEMM
_MIN_TILES = 38
_SMS = 152


def _bn(N: int) -> int:
    """The tensor-core GEMM's tile width for an output N wide."""
    return 64 if N <= 64 else 256


def _tiles(M: int, N: int) -> int:
    """Output tiles of the tensor-core GEMM (128 x 64 when N <= 64, else 128 x 256)."""
    return -(-M // 128) * -(-N // (64 if N <= 64 else 256))


def _wave_eff(units: int) -> float:
    """Busy fraction of the SMs over the rounds a persistent launch of
    ``units`` work units takes (one unit per SM at a time)."""
    return units / (-(-units // _SMS) * _SMS)


# the time model of the K split: a tile's MMA time per 64-wide K block
# (128 x BN x 64 BF16 products at the sustained tensor rate shared by the
# SMs) and the DRAM time of the FP32 partials a split writes and the
# reduction reads back
_TC_SM_RATE = 1.74e15 / _SMS   # flop/s per SM
_HBM_BPS = 6.0e12              # bytes/s


def _ksplit(tiles: int, kp: int, mn: int | None = None, bn: int = 256) -> int:
    """The K split for a GEMM of ``tiles`` output tiles (``bn`` wide), K' =
    kp and ``mn`` outputs: 0 (use the FP32-pair GEMM) when there are few
    tiles and K is short; else the split (slices of at least 8 K blocks)
    that minimises rounds of tiles x slice time + the partials' DRAM time,
    so a split fills idle SMs only where that pays for its partials.
    Without ``mn`` the partials are taken as free."""
    nk = -(-kp // 64)
    if tiles < _MIN_TILES and nk < 16:
        return 0
    t_blk = 2.0 * 128 * bn * 64 / _TC_SM_RATE

    def cost(ks):
        rounds = -(-(tiles * ks) // _SMS)
        part = 0.0 if ks == 1 or mn is None else 8.0 * ks * mn / _HBM_BPS
        return rounds * -(-nk // ks) * t_blk + part
    best, best_t = 1, cost(1)
    for ks in (2, 3, 4, 6, 8, 12, 16, 24, 32, 48, 64, 96, 128, 152):
        if nk // ks < 8:
            break
        t = cost(ks)
        if t < 0.95 * best_t:
            best, best_t = ks, t
    return best


def split_a(A: torch.Tensor) -> torch.Tensor:
    """A' ([hi|hi|lo], K-major) of a 2-D FP64 operand, for reuse through
    ``gemm_tc(..., a_split=)`` when A is a constant integral block."""
    return _split_view(A, A.shape[0], A.shape[1], A.shape[0], 0, A.stride(0), A.stride(1), True, False)


def split_b(B: torch.Tensor) -> torch.Tensor:
    """B' ([hi|lo|hi], rows n, K-major) of a 2-D FP64 operand [K, N], for
    reuse through ``gemm_tc(..., b_split=)``."""
    return _split_view(B, B.shape[1], B.shape[0], B.shape[1], 0, B.stride(1), B.stride(0), False, True)


def gemm_tc(A: torch.Tensor, B: torch.Tensor, C: torch.Tensor, alpha: float = 1.0, beta: float = 0.0,
            status: torch.Tensor | None = None, a_split: torch.Tensor | None = None,
            b_split: torch.Tensor | None = None):
    """C = alpha A @ B + beta C with split-BF16x3 operands on the tcgen05
    tensor cores (FP32 accumulation, FP64 epilogue): the contract of
    ``rccsd_dense.gemm_df`` -- FP64 tensors with any strides, 2-D or batched
    3-D with one operand shared (batch stride 0), flattened into one GEMM.
    Few output tiles with a long K split K; few tiles with a short K, or both
    operands batched, go to ``gemm_df``.  ``status`` (a device int32) makes the launch
    stream-ordered; a gave-up pipeline wait is recorded there.
    ``a_split`` / ``b_split``: the split of a constant 2-D operand made once
    by ``split_a`` / ``split_b``."""
    from . import rccsd_dense as D
    sA, bA = D._strides3(A)
    sB, bB = D._strides3(B)
    sC, batch = D._strides3(C)
    M, N, K = C.shape[-2], C.shape[-1], A.shape[-1]
    assert A.shape[-2] == M and B.shape[-2] == K and B.shape[-1] == N and bA in (1, batch) and bB in (1, batch)
    a_b = batch > 1 and bA > 1 and sA[2] != 0   # batched (an expanded view has batch stride 0)
    b_b = batch > 1 and bB > 1 and sB[2] != 0
    if batch > 1 and a_b == b_b:
        return D.gemm_df(A, B, C, alpha, beta)
    Mf = M * (batch if a_b else 1)
    Nf = N * (batch if b_b else 1)
    # a narrow side goes to N (64-wide tiles): C^T = B^T A^T when M is small
    swap = Mf <= 64 < Nf
    ks = _ksplit(_tiles(Nf, Mf) if swap else _tiles(Mf, Nf), _kp(K), Mf * Nf,
                 _bn(Mf if swap else Nf)) if K > 0 else 0
    if ks == 0:
        return D.gemm_df(A, B, C, alpha, beta)
    # rows of A' are (b, m) or m; rows of B' are (b, n) or n; both K-major
    if a_split is not None:
        assert Mf == M and a_split.shape == (M, _kp(K))
        Ap = a_split
        mi, sro, sri = M, 0, sC[0]
    elif Mf > M:
        Ap = _split_view(A, Mf, K, M, sA[2], sA[0], sA[1], True, False)
        mi, sro, sri = M, sC[2], sC[0]
    else:
        Ap = _split_view(A, M, K, M, 0, sA[0], sA[1], True, False)
        mi, sro, sri = M, 0, sC[0]
    if b_split is not None:
        assert Nf == N and b_split.shape == (N, _kp(K))
        Bp = b_split
        ni, sco, sci = N, 0, sC[1]
    elif Nf > N:
        Bp = _split_view(B, Nf, K, N, sB[2], sB[1], sB[0], False, True)
        ni, sco, sci = N, sC[2], sC[1]
    else:
        Bp = _split_view(B, N, K, N, 0, sB[1], sB[0], False, True)
        ni, sco, sci = N, 0, sC[1]
    kp = Ap.shape[1]
    if swap:  # the operands' split patterns are complementary, so either may sit in the A slot
        Ap, Bp, Mf, Nf = Bp, Ap, Nf, Mf
        mi, sro, sri, ni, sco, sci = ni, sco, sci, mi, sro, sri
    L.check(L.load().fricc_gemm_bf16_tn_strided(_p(Ap), kp, _p(Bp), kp, Mf, Nf, kp, _p(C), mi, ni, sro, sri, sco,
                                                sci, float(alpha), float(beta), ks,
                                                _p(status) if status is not None else None, _st()))
    return C


def dense_spmm_ok(dims, pa, pb, ka, kb, QS: int) -> bool:
    """Whether ``dense_spmm`` takes this term (enough tiles, or a K long
    enough to split)."""
    nP, R = dims[pa] * dims[pb], dims[ka] * dims[kb]
    return _ksplit(_tiles(nP, QS), _kp(R), nP * QS, _bn(QS)) > 0


def dense_spmm(T, dims, pa, pb, ka, kb, coef, Bt: torch.Tensor, QS: int, Op: torch.Tensor,
               status: torch.Tensor | None = None) -> bool:
    """Op[P][q] += coef * sum_r T[P][r] W[r][q] as a dense tensor-core GEMM:
    the compressed T scattered into a zero-filled split-BF16x3 A' (rows
    P = (pa,pb), K = (ka,kb)), Bt = the split W^T ([hi|lo|hi], rows q).
    Returns False (and does nothing) when the GEMM would have too few tiles
    and too short a K for the tensor cores."""
    nP, R = dims[pa] * dims[pb], dims[ka] * dims[kb]
    kp = _kp(R)
    assert Bt.shape == (QS, kp) and Op.is_contiguous() and Op.numel() == nP * QS
    ks = _ksplit(_tiles(nP, QS), kp, nP * QS, _bn(QS))
    if ks == 0:
        return False
    Ap = torch.empty(nP, kp, dtype=torch.bfloat16, device=Op.device)
    lib = L.load()
    L.check(lib.fricc_densify_bf16x3(T, pa, pb, ka, kb, float(coef), _p(Ap), kp, _st()))
    L.check(lib.fricc_gemm_bf16_tn_strided(_p(Ap), kp, _p(Bt), kp, nP, QS, kp, _p(Op), nP, QS, 0, QS, 0, 1,
                                           1.0, 1.0, ks, _p(status) if status is not None else None, _st()))
    return True


def lvv_t(Lf: torch.Tensor, nocc: int) -> torch.Tensor:
    """L_vv^T [v*v, naux] (row c*v + a = L[:, a, c]) of a factor L [naux, nmo, nmo]."""
    naux = Lf.shape[0]
    return Lf[:, nocc:, nocc:].reshape(naux, -1).t().contiguous()


class VvvvRebuild:
    """The (vv|vv) block rebuilt from the split factor: W[(c,d), (a,b)] =
    (ac|bd) in FP32 (rows of ``ldw`` = v*v floats, rounded up to even), on
    demand.  ``rebuild()`` is stream-ordered and capturable: a pipeline wait
    that gave up is recorded in a device status word that ``check()`` reads."""

    def __init__(self, Lf: torch.Tensor, nocc: int):
        nmo = Lf.shape[1]
        self.v = nmo - nocc
        self.Ap, self.Bp = split_bf16x3(lvv_t(Lf, nocc))
        self.kp = self.Ap.shape[1]
        self.ldw = self.v * self.v + (self.v * self.v) % 2
        self.status = torch.zeros(1, dtype=torch.int32, device=Lf.device)
        self.W = None
        self.Bt = None
        self._lock = threading.Lock()
        self.rebuilds = 0

    def flops(self) -> float:
        """Tensor-core flops of one rebuild (the three BF16 products)."""
        return 2.0 * (self.v ** 4) * self.kp

    def rebuild(self, out: torch.Tensor | None = None) -> torch.Tensor:
        """Rebuild into ``out`` (v*v rows of ldw floats), or into the block
        kept on this object (``W``), on the current stream."""
        v = self.v
        if out is not None and (out.dtype != torch.float32 or out.shape != (v * v, self.ldw)
                                or not out.is_contiguous()):
            raise ValueError("out: a contiguous float32 (v*v, ldw) buffer")
        if out is None:
            if self.W is None:
                self.W = torch.empty(v * v, self.ldw, dtype=torch.float32, device=self.Ap.device)
            out = self.W
        L.check(L.load().fricc_vvvv_rebuild_bf16x3(_p(self.Ap), _p(self.Bp), v, self.kp, _p(out), self.ldw,
                                                   _p(self.status), _st()))
        self.rebuilds += 1
        return out

    def rebuild_split_b(self, out: torch.Tensor | None = None) -> torch.Tensor:
        """Rebuild straight into the B operand of the dense O^2V^4 GEMM
        (rows q = (a,b), K = (c,d), [hi | lo | hi]) on the current stream."""
        v = self.v
        kpo = _kp(v * v)
        if out is None:
            out = torch.empty(v * v, kpo, dtype=torch.bfloat16, device=self.Ap.device)
        if out.dtype != torch.bfloat16 or out.shape != (v * v, kpo) or not out.is_contiguous():
            raise ValueError("out: a contiguous bfloat16 (v*v, kp) buffer")
        L.check(L.load().fricc_vvvv_rebuild_split_b(_p(self.Ap), _p(self.Bp), v, self.kp, _p(out), kpo,
                                                    _p(self.status), _st()))
        self.rebuilds += 1
        return out

    def shared_split_b(self) -> torch.Tensor:
        """The B operand rebuilt once and kept on this object for every
        solver of these integrals (built under a lock, then waited for, so
        solvers on other streams and threads read a finished block)."""
        if self.Bt is None:
            with self._lock:
                if self.Bt is None:
                    bt = self.rebuild_split_b()
                    torch.cuda.current_stream().synchronize()
                    self.Bt = bt
        return self.Bt

    def check(self):
        if int(self.status.item()):
            raise L.FriccError(5, "vvvv rebuild: a bounded tensor-core pipeline wait gave up")


def split_eris(system, device="cuda"):
    """DeviceERIs of a synthetic system for the split-precision form: the
    (ov|vv) and (oo|vv) blocks rebuilt from the BF16 hi + lo factor on the
    tensor cores (split-BF16x3, FP32 accumulation, widened to FP64 for the
    dense algebra), the (vv|vv) block never stored in FP64 but rebuilt by
    ``VvvvRebuild`` for the O^2V^4 contraction; the small blocks (oo|oo),
    (ov|oo), (ov|ov) from the FP64 factor on the FP32-pair GEMM (~2^-40),
    (ov|vo) = (ov|ov) permuted (L is symmetric), sum_cd (ac|bd) in FP64."""
    from .rccsd_dense import DeviceERIs, _dev_tensor
    dev = torch.device(device)
    Lf = _dev_tensor(system.L, dev)
    o, nmo = system.nocc, system.nmo
    naux = Lf.shape[0]
    sl = {"o": slice(0, o), "v": slice(o, nmo)}

    def fac(p, q):
        return Lf[:, sl[p], sl[q]].reshape(naux, -1).t().contiguous()  # [(p,q), P]

    def fp64_blk(name):
        # FP64-accurate (~2^-40) on the FP32-pair GEMM: GB300's FP64 unit
        # would spend ~0.1 s per (ov|ov)-sized block of a large request
        from .rccsd_dense import gemm_df
        p, q, r, t = name
        n1 = (Lf[:, sl[p], sl[q]]).shape[1:]
        n2 = (Lf[:, sl[r], sl[t]]).shape[1:]
        A, B = fac(p, q), fac(r, t)
        C = torch.empty(A.shape[0], B.shape[0], dtype=torch.float64, device=dev)
        gemm_df(A, B.t(), C)
        return C.reshape(*n1, *n2)

    def tc_blk(name):
        p, q, r, t = name
        A, _ = split_bf16x3(fac(p, q))
        _, B = split_bf16x3(fac(r, t))
        n1 = (Lf[:, sl[p], sl[q]]).shape[1:]
        n2 = (Lf[:, sl[r], sl[t]]).shape[1:]
        return gemm_bf16_tn(A, B, f64=True).reshape(*n1, *n2)

    blocks = {k: fp64_blk(k) for k in ("oooo", "ovoo", "ovov")}
    blocks["ovvo"] = blocks["ovov"].permute(0, 1, 3, 2).contiguous()  # (ia|bj) = (ia|jb), L symmetric
    blocks["ovvv"] = tc_blk("ovvv")
    blocks["oovv"] = tc_blk("oovv")
    s = Lf[:, o:, o:].sum(dim=2)                      # [P, a] = sum_c L[P,a,c]
    blocks["S0"] = s.t() @ s                          # sum_cd (ac|bd)
    blocks["vvvv_rebuild"] = VvvvRebuild(Lf, o)
    return DeviceERIs(_dev_tensor(system.fock, dev), _dev_tensor(system.mo_energy, dev), o, blocks, device)


# ---------------------------------------------------------------------------
# Replica batches: each replica's GEMM exactly as gemm_tc / dense_spmm run it
# alone (same flattening, swap, K split and tiles), all replicas in one launch
# of the tensor-core kernel.

def _rep_operand(X: torch.Tensor, cdim: int, R: int):
    """(the replica-0 operand as gemm_tc sees it alone, replica stride or 0
    when shared): with a 3-D output [R, M, N] an operand is 3-D (per
    replica) or 2-D (shared); with a 4-D output [R, b, M, N] it is 4-D, per
    replica unless its leading extent is 1 or its leading stride 0."""
    if cdim == 3:
        return (X[0], X.stride(0)) if X.dim() == 3 else (X, 0)
    assert X.dim() == 4, "a 4-D output takes 4-D operands ([1, ...] when shared)"
    shared = X.shape[0] == 1 or X.stride(0) == 0 or R == 1
    return X[0], (0 if shared else X.stride(0))


def gemm_tc_rep(A: torch.Tensor, B: torch.Tensor, C: torch.Tensor, alpha: float, beta: float, R: int,
                status: torch.Tensor | None = None, a_split: torch.Tensor | None = None,
                b_split: torch.Tensor | None = None):
    """gemm_tc(A_r, B_r, C_r) for every replica r = 0..R-1 in one launch:
    C is [R, M, N] or [R, b, M, N]; operands follow ``_rep_operand``.  The
    flattening, the narrow-side swap, the K split and the FP32-pair fallback
    are decided from one replica's shapes, so every replica's result is bit
    for bit that of its own gemm_tc call."""
    from . import rccsd_dense as D
    cdim = C.dim()
    A0, ra = _rep_operand(A, cdim, R)
    B0, rb = _rep_operand(B, cdim, R)
    C0 = C[0]

    def stacked(X, X0, rx):
        # the (replica, batch) rows of a batched per-replica operand must be
        # one stride apart: copy X when its replicas are not stacked so
        s0, bx = D._strides3(X0)
        if rx and bx > 1 and s0[2] != 0 and rx != bx * s0[2]:
            Xc = torch.empty(X.shape, dtype=X.dtype, device=X.device)
            D.combine([Xc], [X])
            return Xc, Xc[0], Xc.stride(0)
        return X, X0, rx
    A, A0, ra = stacked(A, A0, ra)
    B, B0, rb = stacked(B, B0, rb)
    sA, bA = D._strides3(A0)
    sB, bB = D._strides3(B0)
    sC, batch = D._strides3(C0)
    M, N, K = C0.shape[-2], C0.shape[-1], A0.shape[-1]
    assert A0.shape[-2] == M and B0.shape[-2] == K and B0.shape[-1] == N and bA in (1, batch) and bB in (1, batch)
    a_b = batch > 1 and bA > 1 and sA[2] != 0
    b_b = batch > 1 and bB > 1 and sB[2] != 0

    def df():  # the FP32-pair GEMM, every replica as the second batch level
        def four(X, Xr, lone):
            if cdim == 4:
                return X
            return X.unsqueeze(1) if Xr else lone.unsqueeze(0).unsqueeze(0)
        return D.gemm_df(four(A, ra, A0), four(B, rb, B0), C if cdim == 4 else C.unsqueeze(1), alpha, beta)

    if batch > 1 and a_b == b_b:
        df()
        return C
    Mf = M * (batch if a_b else 1)
    Nf = N * (batch if b_b else 1)
    swap = Mf <= 64 < Nf
    ks = _ksplit(_tiles(Nf, Mf) if swap else _tiles(Mf, Nf), _kp(K), Mf * Nf,
                 _bn(Mf if swap else Nf)) if K > 0 else 0
    if ks == 0:
        df()
        return C
    # A' rows: (replica, batch, m) or (replica, m); one split for a shared A
    if a_split is not None:
        assert ra == 0 and Mf == M and a_split.shape == (M, _kp(K))
        Ap, a_rep = a_split, 0
        mi, sro, sri = M, 0, sC[0]
    else:
        if ra:
            Ap = _split_view(A0, R * Mf, K, M, sA[2] if a_b else ra, sA[0], sA[1], True, False)
        else:
            Ap = _split_view(A0, Mf, K, M, sA[2] if a_b else 0, sA[0], sA[1], True, False)
        a_rep = Mf if ra else 0
        mi, sro, sri = M, (sC[2] if a_b else 0), sC[0]
    if b_split is not None:
        assert rb == 0 and Nf == N and b_split.shape == (N, _kp(K))
        Bp, b_rep = b_split, 0
        ni, sco, sci = N, 0, sC[1]
    else:
        if rb:
            Bp = _split_view(B0, R * Nf, K, N, sB[2] if b_b else rb, sB[1], sB[0], False, True)
        else:
            Bp = _split_view(B0, Nf, K, N, sB[2] if b_b else 0, sB[1], sB[0], False, True)
        b_rep = Nf if rb else 0
        ni, sco, sci = N, (sC[2] if b_b else 0), sC[1]
    kp = Ap.shape[1]
    if swap:
        Ap, Bp, Mf, Nf, a_rep, b_rep = Bp, Ap, Nf, Mf, b_rep, a_rep
        mi, sro, sri, ni, sco, sci = ni, sco, sci, mi, sro, sri
    L.check(L.load().fricc_gemm_bf16_tn_strided_b(_p(Ap), kp, _p(Bp), kp, Mf, Nf, kp, _p(C), mi, ni, sro, sri, sco,
                                                  sci, float(alpha), float(beta), ks, R, a_rep, b_rep, C.stride(0),
                                                  _p(status) if status is not None else None, _st()))
    return C


def dense_spmm_rep(spb, which: int, R: int, dims, pa, pb, ka, kb, coef, Bt: torch.Tensor, b_rep: int, QS: int,
                   Op: torch.Tensor, status: torch.Tensor | None = None) -> bool:
    """dense_spmm for every replica of a compressed batch (``spb``, a
    fricc_spbatch handle; compression ``which``) in one densify and one
    tensor-core launch: replica r's A' rows r nP.., its W^T split at row
    r b_rep of Bt (b_rep 0: one W for all), its output Op[r] ([R, nP*QS]
    contiguous).  False (nothing done) where dense_spmm would decline."""
    nP, Rk = dims[pa] * dims[pb], dims[ka] * dims[kb]
    kp = _kp(Rk)
    assert Bt.shape[1] == kp and Bt.shape[0] >= QS and Op.is_contiguous() and Op.numel() == R * nP * QS
    ks = _ksplit(_tiles(nP, QS), kp, nP * QS, _bn(QS))
    if ks == 0:
        return False
    Ap = torch.empty(R * nP, kp, dtype=torch.bfloat16, device=Op.device)
    lib = L.load()
    L.check(lib.fricc_spb_densify_bf16x3(spb, which, pa, pb, ka, kb, float(coef), _p(Ap), kp, _st()))
    L.check(lib.fricc_gemm_bf16_tn_strided_b(_p(Ap), kp, _p(Bt), kp, nP, QS, kp, _p(Op), nP, QS, 0, QS, 0, 1, 1.0,
                                             1.0, ks, R, nP, b_rep, nP * QS,
                                             _p(status) if status is not None else None, _st()))
    return True


def split_b_rep(W: torch.Tensor, R: int, QS: int) -> torch.Tensor:
    """split_b(W[r].reshape(-1, QS)) of every replica, stacked: rows
    (r, q), R*QS of them (W contiguous [R, ...])."""
    assert W.is_contiguous()
    krows = W[0].numel() // QS
    return _split_view(W, R * QS, krows, QS, krows * QS, 1, QS, False, True)
