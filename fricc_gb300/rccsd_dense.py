"""Dense closed-shell CCSD pieces of one FRI-CCSD iteration, on the GPU (FP64).

These are the parts of fricc/friccsd.py:update_amps that the reference
delegates to PySCF (``rintermediates`` cc_Foo, cc_Fvv, cc_Fov, Loo, Lvv and
the dense W intermediates, the CCSD energy) written from the closed-shell
CCSD equations (Hirata et al., J. Chem. Phys. 120, 2581 (2004)), with torch
tensors on the device.  The reference-shaped helpers below (cc_Foo, Loo,
cc_Woooo, ...) are written with torch einsums and serve the uncompressed
variants and the tests; the iteration itself (fricc_gb300.friccsd) runs its
dense algebra on the library's GEMMs (gemm_f64, gemm_df, the tensor-core
GEMM) and its elementwise passes on the library's combine kernel.

Integral blocks, chemists' notation: ovov[i,a,j,b] = (ia|jb),
oovv[i,j,a,b] = (ij|ab), ovvo[i,a,b,j] = (ia|bj), ovoo[i,a,j,k] = (ia|jk),
ovvv[i,a,b,c] = (ia|bc), oooo[i,j,k,l] = (ij|kl); the vvvv block is kept
only as vvvvT[c,d,a,b] = (ac|bd), the layout the O^2V^4 term streams.
"""
from __future__ import annotations

import math

import threading

import numpy as np
import torch

from . import _lib as L

ein = torch.einsum


class DeviceERIs:
    """Integrals and orbital energies resident in HBM for the whole solve."""

    def __init__(self, fock, mo_energy, nocc, blocks, device="cuda"):
        dev = torch.device(device)
        f64 = torch.float64

        def put(a):
            return (a if isinstance(a, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(a))).to(
                dev, f64).contiguous()

        self.device = dev
        self.nocc = int(nocc)
        self.fock = put(fock)
        self.mo_energy = put(mo_energy)
        for k in ("oooo", "ovoo", "ovov", "oovv", "ovvo", "ovvv"):
            setattr(self, k, put(blocks[k]))
        vvvv = put(blocks["vvvv"]) if "vvvv" in blocks else None
        if "vvvvT" in blocks:
            self.vvvvT = put(blocks["vvvvT"])
        elif vvvv is not None:
            self.vvvvT = vvvv.permute(1, 3, 0, 2).contiguous()  # [c,d,a,b] = (ac|bd)
        else:
            # split precision: (vv|vv) is rebuilt from the factor when needed
            # (fricc_gb300.cholesky); only sum_cd (ac|bd) is kept
            self.vvvvT = None
        del vvvv
        self._S0 = put(blocks["S0"]) if "S0" in blocks else None
        self.vvvv_rebuild = blocks.get("vvvv_rebuild")
        self._derive()

    def _derive(self):
        """Constant layouts and combinations reused every iteration."""
        ovvv, ovov, ovoo = self.ovvv, self.ovov, self.ovoo
        self.g_ovov = 2.0 * ovov - ovov.permute(0, 3, 2, 1)               # 2(kc|ld) - (kd|lc)
        self.g_ovoo = 2.0 * ovoo - ovoo.permute(2, 1, 0, 3)               # [l,c,k,i]: 2(lc|ki) - (kc|li)
        # T1 O^2V^3 terms as one GEMM: G[k,c,d,a] = 2 (kd|ac) - (kc|ad)
        self.G_t1 = (2.0 * ovvv.permute(0, 3, 1, 2) - ovvv.permute(0, 1, 3, 2)).contiguous()
        # the same integral as [k,d,c,a]: X[c,a] = sum_kd t1[k,d] G[k,c,d,a] is one GEMV
        # (it serves the t1.t1 T1 term and the ovvv part of Lvv)
        self.G_t1_kdca = self.G_t1.permute(0, 2, 1, 3).contiguous()
        # the T1 terms 2 sum_kc (kc|ai) t_kc - sum_kc (ki|ac) t_kc as one GEMV:
        # G1[k,c,i,a] = 2 (kc|ai) - (ki|ac)
        self.G_t1_kcia = (2.0 * self.ovvo.permute(0, 1, 3, 2) - self.oovv.permute(0, 3, 1, 2)).contiguous()
        # the t1 parts of Wvvvv, contracted with the compressed T2 instead of being
        # built densely: W'[c,d,(x,k,a)] = (kd|ac) for x=0 and (kc|ad) for x=1
        self.ovvv_XY = torch.stack([ovvv.permute(3, 1, 0, 2), ovvv.permute(1, 3, 0, 2)], dim=2).contiguous()
        # sum_cd of the three Wvvvv pieces (for the reference's Wvvvv.t1.t1 term)
        self.S0 = self._S0 if self._S0 is not None else self.vvvvT.sum(dim=(0, 1))  # [a,b] = sum_cd (ac|bd)
        self.U = ovvv.sum(dim=(1, 3))                                     # [k,a] = sum_cd (kd|ac) = sum_cd (kc|ad)
        # W' of the sparse W-intermediate terms, [l,d,k,c]
        self.ovov_0312 = ovov.permute(0, 3, 2, 1).contiguous()            # (lc|kd)
        self.ovov_0313_0113 = (ovov - 0.5 * ovov.permute(0, 3, 2, 1)).contiguous()
        self.ovov_cdkl = ovov.permute(1, 3, 0, 2).contiguous()            # 1323: [c,d,k,l] = (kc|ld)
        # GEMM-ready layouts for the dense O^2V^3 contractions
        self.g_klcd = self.g_ovov.permute(0, 2, 1, 3).contiguous()       # cc_Foo
        self.g_kldc = self.g_ovov.permute(0, 2, 3, 1).contiguous()       # cc_Fvv
        self.ovvv_iabc = ovvv.permute(0, 1, 3, 2).contiguous()           # T2 driver term
        self.ovvv_kacd = ovvv.permute(0, 2, 3, 1).contiguous()           # Wvovo t1 term
        self._dense_wvvvv = None
        self._splits = {}
        self._lock = threading.Lock()

    SPLIT_BLOCKS = ("vvvvT", "ovvv_XY", "ovov", "ovov_0312", "ovov_0313_0113", "ovov_cdkl")

    def prepare_splits(self, names=None):
        """Build the (hi, lo) float-pair forms of constant W' blocks once (by
        default those of FRI-CCSD), and wait for them: solvers on other
        streams read them afterwards."""
        names = self.SPLIT_BLOCKS if names is None else names
        if any(n not in self._splits for n in names):
            for name in names:
                if name not in self._splits and getattr(self, name) is not None:
                    self._splits[name] = split_f2(getattr(self, name))
            torch.cuda.current_stream().synchronize()

    LIN_BLOCKS = ("oooo_klij", "lin_WA", "lin_WB", "lin_W2AB")

    def prepare_linear(self):
        """The bare-integral W' layouts FRI-LCCSD contracts the compressed T2
        with (fricc/frilccsd.py:172-175), built once and shared by solvers:
        oooo_klij[k,l,i,j] = (ki|lj) (0101), lin_WA[k,c,i,a] = (kc|ai)
        (1302, 1303), lin_WB[k,c,i,a] = (ki|ac) (1202, 1203) and
        2 lin_WA - lin_WB (1302 and 1202 from one compression)."""
        if not hasattr(self, "lin_WA"):
            self.oooo_klij = self.oooo.permute(0, 2, 1, 3).contiguous()
            self.lin_WA = self.ovvo.permute(0, 1, 3, 2).contiguous()
            self.lin_WB = self.oovv.permute(0, 3, 1, 2).contiguous()
            self.lin_W2AB = (2.0 * self.lin_WA - self.lin_WB).contiguous()
            if self.device.type == "cuda":
                torch.cuda.current_stream().synchronize()

    def prepare_f32(self, blocks: dict):
        """Build the FP32 forms {name: qs} once, and wait for them (solvers
        on other streams read them afterwards)."""
        if any(("f32", n, q) not in self._splits for n, q in blocks.items()):
            for n, q in blocks.items():
                self.f32(n, q)
            torch.cuda.current_stream().synchronize()

    def prepare_tc(self, operands: dict):
        """The split-BF16x3 operands of constant blocks for the split-precision
        form's tensor-core GEMMs, made once and waited for:
        {name: ("A" or "B", rows, cols)} with the block viewed as [rows, cols]."""
        from .cholesky import split_a, split_b
        todo = {n: spec for n, spec in operands.items() if ("tc", n) not in self._splits}
        if todo:
            for n, (role, r, c) in todo.items():
                x = getattr(self, n).reshape(r, c)
                self._splits[("tc", n)] = (role, split_a(x) if role == "A" else split_b(x))
            torch.cuda.current_stream().synchronize()

    def tc_w(self, name, qs):
        """The split W^T ([hi|lo|hi], rows q) of a constant W' block viewed as
        [rows][qs]: the B operand of the split-precision dense sparse terms.
        Built on first use (the first, eager iteration) under a lock and
        waited for, so solvers on other threads and streams never read a
        block whose split is still in flight."""
        from .cholesky import split_b
        key = ("tcW", name, qs)
        got = self._splits.get(key)
        if got is None:
            with self._lock:
                got = self._splits.get(key)
                if got is None:
                    got = split_b(getattr(self, name).reshape(-1, qs))
                    torch.cuda.current_stream().synchronize()
                    self._splits[key] = got
        return got

    def tc(self, name, role):
        got = self._splits.get(("tc", name))
        if got is None or got[0] != role:
            raise RuntimeError(f"split operand {role} of {name} missing: call prepare_tc() first")
        return got[1]

    def f32(self, name, qs):
        """FP32 rows (qs columns, padded to even) of a constant block, built
        once: the W' operands of the split-precision form."""
        key = ("f32", name, qs)
        if key not in self._splits:
            self._splits[key] = to_f32_rows(getattr(self, name), qs)
        return self._splits[key]

    def split(self, name):
        """The float-pair form of a constant block (prepare_splits() built it)."""
        if name not in self._splits:
            raise RuntimeError(f"float-pair form of {name} missing: call prepare_splits() first")
        return self._splits[name]

    @property
    def ovvv_kcda(self):  # [k,c,d,a] = (kd|ac), only for the dense Wvvvv build
        return self.ovvv.permute(0, 3, 1, 2).contiguous()

    @property
    def ovvv_cdkb(self):  # [c,d,k,b] = (kc|bd), only for the dense Wvvvv build
        return self.ovvv.permute(1, 3, 0, 2).contiguous()

    @classmethod
    def from_system(cls, system, device="cuda"):
        """Build every block on the device from the Cholesky factor of a SyntheticSystem."""
        dev = torch.device(device)
        L = _dev_tensor(system.L, dev)
        o = system.nocc
        naux = L.shape[0]
        sl = {"o": slice(0, o), "v": slice(o, system.nmo)}

        def blk(name):
            p, q, r, s = (sl[c] for c in name)
            A = L[:, p, q].reshape(naux, -1)
            B = L[:, r, s].reshape(naux, -1)
            n1 = L[:, p, q].shape[1:]
            n2 = L[:, r, s].shape[1:]
            return (A.T @ B).reshape(*n1, *n2)

        blocks = {k: blk(k) for k in ("oooo", "ovoo", "ovov", "oovv", "ovvv")}
        # (ia|bj) = (ia|jb): L is symmetric in its two orbital indices
        blocks["ovvo"] = blocks["ovov"].permute(0, 1, 3, 2).contiguous()
        Lvv = L[:, sl["v"], sl["v"]]
        v = system.nvir
        # vvvvT[c,d,a,b] = (ac|bd) = sum_P L[P,a,c] L[P,b,d]
        Lca = Lvv.permute(0, 2, 1).reshape(naux, v * v)  # [P, (c,a)]
        Ldb = Lvv.permute(0, 2, 1).reshape(naux, v * v)  # [P, (d,b)]
        X = (Lca.T @ Ldb).reshape(v, v, v, v)            # [c,a,d,b]
        blocks["vvvvT"] = X.permute(0, 2, 1, 3).contiguous()
        del X
        return cls(_dev_tensor(system.fock, dev), _dev_tensor(system.mo_energy, dev), o, blocks, device)

    def to_numpy_blocks(self):
        """Host copies in the stand-in layout (for checking against the oracle)."""
        out = {k: getattr(self, k).cpu().numpy() for k in ("oooo", "ovoo", "ovov", "oovv", "ovvo", "ovvv")}
        out["vvvv"] = self.vvvvT.permute(2, 0, 3, 1).contiguous().cpu().numpy()  # (ab|cd)
        return out


def sym_add(out: torch.Tensor, X: torch.Tensor, coef: float = 1.0) -> torch.Tensor:
    """out += coef * (X + X.permute(1, 0, 3, 2)) in one fused pass (the
    symmetrised T2 residual terms); out contiguous [o,o,v,v] FP64 on the
    device, X any [o,o,v,v] FP64 view not overlapping out."""
    import ctypes

    o, v = out.shape[0], out.shape[2]
    if (not out.is_contiguous() or out.dtype != torch.float64 or X.dtype != torch.float64
            or tuple(X.shape) != tuple(out.shape) or out.shape != (o, o, v, v)):
        raise ValueError("sym_add: out contiguous [o,o,v,v] float64 and X a float64 view of the same shape")
    L.check(L.load().fricc_symadd(ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(X.data_ptr()), o, v,
                                  L.i64arr(X.stride()), float(coef),
                                  L.cur_stream()))
    return out


def _view5(t: torch.Tensor, shape):
    """Element strides of ``t`` broadcast to ``shape``, padded to 5 dims."""
    b = t.expand(*shape) if tuple(t.shape) != tuple(shape) else t
    st = list(b.stride())
    return [0] * (5 - len(st)) + st


def combine(outs, xs=(), coefs=None, prod=(), accumulate=False):
    """One pass of the library's strided elementwise kernel (fricc_combine5):
    out_k = sum_t coefs[k][t] xs[t] (+ coefs[k][-1] * prod[0] * prod[1] ...
    when ``prod`` is given), or out_k += that with ``accumulate``.  Every
    tensor is an FP64 device view; inputs broadcast to the outputs' shape
    (at most 5 dims); the kernel walks the first output's memory order.
    Outputs must not overlap the inputs."""
    import ctypes

    outs = list(outs)
    xs = list(xs)
    prod = list(prod)
    shape = tuple(outs[0].shape)
    if len(shape) > 5 or any(tuple(o.shape) != shape for o in outs):
        raise ValueError("combine: outputs of one shape, at most 5 dims")
    for t in outs + xs + prod:
        if t.dtype != torch.float64 or t.device.type != "cuda":
            raise ValueError("combine: FP64 CUDA tensors only")
    nc = len(xs) + (1 if prod else 0)
    if coefs is None:
        coefs = [[1.0] * nc for _ in outs]
    if len(coefs) != len(outs) or any(len(c) != nc for c in coefs):
        raise ValueError("combine: one coefficient per input (and one for the product) per output")
    dims = [1] * (5 - len(shape)) + list(shape)
    vp = ctypes.c_void_p

    def ptrs(ts):
        return (vp * max(len(ts), 1))(*[t.data_ptr() for t in ts])

    # walk the index space in the first output's memory order (its
    # smallest stride innermost), so its reads and writes coalesce
    s0 = _view5(outs[0], shape)
    perm = sorted(range(5), key=lambda d: (dims[d] != 1, -s0[d]))

    def strides(ts):
        flat = []
        for t in ts:
            st = _view5(t, shape)
            flat.extend(st[d] for d in perm)
        return L.i64arr(flat if flat else [0])

    cf = (ctypes.c_double * (len(outs) * nc))(*[float(c) for row in coefs for c in row])
    L.check(L.load().fricc_combine5(L.i64arr([dims[d] for d in perm]), len(xs), ptrs(xs), strides(xs), len(prod),
                                    ptrs(prod), strides(prod), len(outs), ptrs(outs), strides(outs), cf,
                                    int(bool(accumulate)), L.cur_stream()))
    return outs[0]


def zero(t: torch.Tensor) -> torch.Tensor:
    """t[...] = 0 for a contiguous device tensor, through the library."""
    import ctypes

    if not t.is_contiguous():
        raise ValueError("zero: contiguous tensors only")
    L.check(L.load().fricc_zero(ctypes.c_void_p(t.data_ptr()), t.numel() * t.element_size(),
                                L.cur_stream()))
    return t


def _dev_tensor(a, dev):
    """FP64 copy of a numpy array, or the tensor itself moved to ``dev``."""
    t = a if isinstance(a, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(a))
    return t.to(dev, torch.float64)


def _strides3(t: torch.Tensor):
    if t.dim() == 2:
        return (t.stride(0), t.stride(1), 0), 1
    return (t.stride(1), t.stride(2), t.stride(0)), t.shape[0]


def _bstrides(t: torch.Tensor):
    """(row, col, batch, batch2) element strides and (batch, batch2) extents of
    a 2-D, 3-D ([batch, M, K]) or 4-D ([batch2, batch, M, K]) operand."""
    if t.dim() == 2:
        return (t.stride(0), t.stride(1), 0, 0), 1, 1
    if t.dim() == 3:
        return (t.stride(1), t.stride(2), t.stride(0), 0), t.shape[0], 1
    if t.dim() == 4:
        return (t.stride(2), t.stride(3), t.stride(1), t.stride(0)), t.shape[1], t.shape[0]
    raise ValueError("gemm: operands are 2-D, 3-D or 4-D")


def _gemm_call(fn, A, B, C, alpha, beta):
    import ctypes

    sA, bA, b2A = _bstrides(A)
    sB, bB, b2B = _bstrides(B)
    sC, batch, batch2 = _bstrides(C)
    M, N = C.shape[-2], C.shape[-1]
    K = A.shape[-1]
    assert A.shape[-2] == M and B.shape[-2] == K and B.shape[-1] == N
    assert bA in (1, batch) and bB in (1, batch) and b2A in (1, batch2) and b2B in (1, batch2)
    # a size-1 batch level of an operand is shared: stride 0
    sA = (sA[0], sA[1], sA[2] if bA == batch and batch > 1 else 0, sA[3] if b2A == batch2 and batch2 > 1 else 0)
    sB = (sB[0], sB[1], sB[2] if bB == batch and batch > 1 else 0, sB[3] if b2B == batch2 and batch2 > 1 else 0)
    lib = L.load()
    st = L.cur_stream()
    pA, pB, pC = (ctypes.c_void_p(t.data_ptr()) for t in (A, B, C))
    if batch2 == 1:
        L.check(getattr(lib, fn)(pA, pB, pC, batch, M, N, K, L.i64arr(sA[:3]), L.i64arr(sB[:3]), L.i64arr(sC[:3]),
                                 float(alpha), float(beta), st))
    else:
        L.check(getattr(lib, fn + "_b2")(pA, pB, pC, batch, batch2, M, N, K, L.i64arr(sA), L.i64arr(sB),
                                         L.i64arr(sC), float(alpha), float(beta), st))
    return C


def gemm_df(A: torch.Tensor, B: torch.Tensor, C: torch.Tensor, alpha: float = 1.0, beta: float = 0.0):
    """C = alpha A @ B + beta C on the FP32-pair GEMM kernel; FP64 tensors with
    any strides, 2-D or batched 3-D (a batch stride of 0 shares an operand)."""
    return _gemm_call("fricc_gemm_df", A, B, C, alpha, beta)


def gemm_f64(A: torch.Tensor, B: torch.Tensor, C: torch.Tensor, alpha: float = 1.0, beta: float = 0.0):
    """The same contract in FP64 on the library's DFMA GEMM kernel."""
    return _gemm_call("fricc_gemm_f64", A, B, C, alpha, beta)


def _as3(x: torch.Tensor, shape3):
    """x (a permuted view) as a [batch, rows, cols] view, copied to a
    contiguous buffer by the library when its strides do not allow one."""
    try:
        return x.view(*shape3)
    except RuntimeError:
        if x.device.type != "cuda":
            return x.reshape(*shape3)
        buf = torch.empty(x.shape, dtype=x.dtype, device=x.device)
        combine([buf], [x])
        return buf.view(*shape3)


def einsum_df(spec: str, A: torch.Tensor, B: torch.Tensor, gemm=None, out=None, alpha: float = 1.0,
              beta: float = 0.0) -> torch.Tensor:
    """Two-operand einsum as one strided batched GEMM on the FP32-pair kernel.

    Indices shared by both operands and the output form the batch, A-only
    output indices the rows, B-only output indices the columns, shared
    non-output indices the contraction; an index in one operand only and not
    in the output is summed out first.  ``gemm`` replaces the FP32-pair GEMM
    (the FP64 form passes the DFMA one, the split-precision form the
    tensor-core one).  Operand groups merge into one stride where the layout
    allows (the library copies them otherwise).  Without ``out`` the result
    is a view of a new contiguous [batch, rows, cols] buffer in the output's
    order; with ``out`` (a tensor in the output's index order whose
    [batch, rows, cols] grouping is a view) the GEMM writes
    out = alpha * result + beta * out in place."""
    lhs, outs = spec.replace(" ", "").split("->")
    a, b = lhs.split(",")
    if len(set(a)) != len(a) or len(set(b)) != len(b):
        raise ValueError(f"einsum_df: repeated index within an operand in {spec!r}")
    lone = [c for c in a if c not in b and c not in outs]
    if lone:
        A = A.sum(dim=[a.index(c) for c in lone])
        a = "".join(c for c in a if c not in lone)
    lone = [c for c in b if c not in a and c not in outs]
    if lone:
        B = B.sum(dim=[b.index(c) for c in lone])
        b = "".join(c for c in b if c not in lone)
    size = {c: A.shape[a.index(c)] for c in a}
    size.update({c: B.shape[b.index(c)] for c in b})
    bt = [c for c in outs if c in a and c in b]
    mi = [c for c in outs if c in a and c not in b]
    ni = [c for c in outs if c in b and c not in a]
    ki = [c for c in a if c in b and c not in outs]
    prod = lambda idx: math.prod(size[c] for c in idx)
    nb, M, N, K = prod(bt), prod(mi), prod(ni), prod(ki)
    Ap = _as3(A.permute([a.index(c) for c in bt + mi + ki]), (nb, M, K))
    Bp = _as3(B.permute([b.index(c) for c in bt + ki + ni]), (nb, K, N))
    order = bt + mi + ni
    if out is not None:
        C = out.permute([outs.index(c) for c in order]).view(nb, M, N)
    else:
        C = torch.empty(nb, M, N, dtype=torch.float64, device=A.device)
        alpha, beta = 1.0, 0.0
    if C.numel():
        if K == 0:
            if beta == 0.0:
                C.zero_()
        else:
            (gemm or gemm_df)(Ap, Bp, C, alpha, beta)
    if out is not None:
        return out
    return C.view([size[c] for c in order]).permute([order.index(c) for c in outs])


def gemm_torch(A, B, C, alpha=1.0, beta=0.0):
    """The same contract on cuBLAS FP64."""
    R = torch.matmul(A, B)
    if beta == 0.0:
        C.copy_(R.mul_(alpha) if alpha != 1.0 else R)
    else:
        if beta != 1.0:
            C.mul_(beta)
        C.add_(R, alpha=alpha)
    return C


def to_f32_rows(x: torch.Tensor, qs: int) -> torch.Tensor:
    """x viewed as [rows][qs] in FP32, rows padded to an even length (the
    layout fricc_spmm_f1 reads as float pairs)."""
    rows = x.numel() // qs
    x2 = x.reshape(rows, qs)
    if qs % 2 == 0:
        return x2.to(torch.float32).contiguous()
    out = torch.zeros(rows, qs + 1, dtype=torch.float32, device=x.device)
    out[:, :qs] = x2
    return out


def split_f2(x: torch.Tensor, qs: int = None) -> torch.Tensor:
    """W' [rows][qs] (FP64) as float pairs hi + lo = x (to 2^-47), in the
    q-pair layout of fricc_spmm_f2: per row, float4 (hi_q, hi_q+1, lo_q,
    lo_q+1) for q = 0, 2, 4, ...  qs defaults to the product of the
    dimensions after the first two (W' is always [key1, key2, q...])."""
    import ctypes

    x = x.contiguous()
    if qs is None:
        qs = math.prod(x.shape[2:]) if x.dim() > 2 else x.shape[-1]
    rows = x.numel() // qs
    out = torch.empty(rows * ((qs + 1) // 2) * 4, dtype=torch.float32, device=x.device)
    L.check(L.load().fricc_split_f2(ctypes.c_void_p(x.data_ptr()), rows, qs, ctypes.c_void_p(out.data_ptr()),
                                    L.cur_stream()))
    return out


def cc_Foo(t1, t2, E):
    o = t1.shape[0]
    tt = t2 + ein("ic,ld->ilcd", t1, t1)
    return E.fock[:o, :o] + ein("kcld,ilcd->ki", E.g_ovov, tt)


def cc_Fvv(t1, t2, E):
    o = t1.shape[0]
    tt = t2 + ein("ka,ld->klad", t1, t1)
    return E.fock[o:, o:] - ein("kcld,klad->ac", E.g_ovov, tt)


def cc_Fov(t1, t2, E):
    o = t1.shape[0]
    return E.fock[:o, o:] + ein("kcld,ld->kc", E.g_ovov, t1)


def Loo(t1, t2, E, Foo=None):
    o = t1.shape[0]
    fov = E.fock[:o, o:]
    F = cc_Foo(t1, t2, E) if Foo is None else Foo
    return F + fov @ t1.T + ein("lcki,lc->ki", E.g_ovoo, t1)


def Lvv(t1, t2, E, Fvv=None):
    o = t1.shape[0]
    fov = E.fock[:o, o:]
    F = cc_Fvv(t1, t2, E) if Fvv is None else Fvv
    return F - t1.T @ fov + 2.0 * ein("kdac,kd->ac", E.ovvv, t1) - ein("kcad,kd->ac", E.ovvv, t1)


def cc_Woooo(t1, t2, E):
    W = ein("lcki,jc->klij", E.ovoo, t1)
    W = W + ein("kclj,ic->klij", E.ovoo, t1)
    W = W + ein("kcld,ijcd->klij", E.ovov, t2 + ein("ic,jd->ijcd", t1, t1))
    return W + E.oooo.permute(0, 2, 1, 3)


def cc_Wvoov(t1, t2, E):
    W = ein("kcad,id->akic", E.ovvv, t1)
    W = W - ein("kcli,la->akic", E.ovoo, t1)
    W = W + E.ovvo.permute(2, 0, 3, 1)
    W = W - 0.5 * ein("ldkc,ilda->akic", E.ovov, t2)
    W = W - 0.5 * ein("lckd,ilad->akic", E.ovov, t2)
    W = W + ein("ldkc,ilad->akic", E.ovov, t2)
    return W - ein("ldkc,id,la->akic", E.ovov, t1, t1)


def cc_Wvovo(t1, t2, E):
    W = ein("kdac,id->akci", E.ovvv, t1)
    W = W - ein("lcki,la->akci", E.ovoo, t1)
    W = W + E.oovv.permute(2, 0, 3, 1)
    W = W - 0.5 * ein("lckd,ilda->akci", E.ovov, t2)
    return W - ein("lckd,id,la->akci", E.ovov, t1, t1)


def wvvvv_T(t1, E, out=None):
    """Wvvvv of fricc/friccsd.py:325-331 in the streamed layout [c,d,a,b]:
    (ac|bd) - sum_k (kd|ac) t_kb - sum_k (kc|bd) t_ka."""
    o, v = t1.shape
    W = E.vvvvT.clone() if out is None else out.copy_(E.vvvvT)
    Wf = W.view(v * v, v, v)  # [(c,d), a, b]
    # - sum_k (kd|ac) t_kb  ->  [c,d,a] x [k] . [k,b]
    Wf.view(v * v * v, v).addmm_(E.ovvv_kcda.view(o, v * v * v).T, t1, alpha=-1.0)
    # - sum_k (kc|bd) t_ka  ->  per (c,d): t1^T [a,k] @ (kc|bd)[k,b]
    Wf.baddbmm_(t1.T.unsqueeze(0).expand(v * v, v, o), E.ovvv_cdkb.view(v * v, o, v), alpha=-1.0)
    return W


def wvvvv_sum_cd(t1, E):
    """S[a,b] = sum_cd Wvvvv[a,b,c,d] without building Wvvvv:
    sum_cd (ac|bd) - sum_k t_kb sum_cd (kd|ac) - sum_k t_ka sum_cd (kc|bd)."""
    return E.S0 - E.U.T @ t1 - t1.T @ E.U


def lin_cc_energy(t1, t2, E):
    """2 sum f_ia t1_ia + sum t2_ijab (2 (ia|jb) - (ib|ja)) (fricc/frilccsd.py:504-522)."""
    o = t1.shape[0]
    fov = E.fock[:o, o:]
    return float(2.0 * (fov * t1).sum() + ein("ijab,iajb->", t2, E.g_ovov))


def ccsd_energy(t1, t2, E):
    o = t1.shape[0]
    fov = E.fock[:o, o:]
    tau = t2 + ein("ia,jb->ijab", t1, t1)
    return float(2.0 * (fov * t1).sum() + ein("ijab,iajb->", tau, E.g_ovov))
