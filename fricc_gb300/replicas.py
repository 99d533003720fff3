"""Replica batches with one launch per kernel for all replicas.

R independent FRI-CCSD replicas of one system (distinct seeds, shared
integrals) run as one stacked iteration: amplitudes t1 [R, o, v] and
t2 [R, o, o, v, v], every kernel of fricc/friccsd.py:update_amps launched
once with the replica as one more grid dimension -- both FRI compressions
of every replica (fricc/friccsd.py:100-117) in one batched paired
compression, every sparse term in one batched launch, the dense GEMMs with
the replica as a second batch level, every elementwise pass over a 5-D index
space, the energy of every replica in one launch.  Each replica's arithmetic
is that of its own ``FRICCSDGPU`` iteration (the same kernels, tiles, K
splits and summation orders), so each replica's trajectory is bit for bit
the one its lone solve gives with the same seed.

The replicas' statistics are those of fricc/__init__.py:8-11 (``mcmc_std``
of each trace; the replica mean and variance of E_corr).
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _lib as L
from . import rccsd_dense as D
from .rng import GlibcRand

ALL_TERMS = ["O^2V^4", "O^3V^3", "O^4V^2"]


def _ptr(t: torch.Tensor) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr())


def _as4(x: torch.Tensor, shape4):
    """x as a [R, batch, rows, cols] view, copied by the library when its
    strides do not allow one (as einsum_df copies a single replica's)."""
    try:
        return x.view(*shape4)
    except RuntimeError:
        if x.device.type != "cuda":
            return x.reshape(*shape4)
        buf = torch.empty(x.shape, dtype=x.dtype, device=x.device)
        D.combine([buf], [x])
        return buf.view(*shape4)


def einsum_rep(spec: str, A: torch.Tensor, B: torch.Tensor, gemm, za: bool, zb: bool, R: int, out=None,
               alpha: float = 1.0, beta: float = 0.0):
    """einsum_df(spec, A_r, B_r) for every replica r at once: ``spec`` is the
    single-replica contraction; A (B) carries a leading replica dimension
    when ``za`` (``zb``), else it is shared.  Each replica's operands are
    grouped, copied and multiplied exactly as einsum_df does for one
    replica (the replica is the GEMM's second batch level), so the results
    are bit for bit the single calls'.  With ``out`` (shape [R, ...out],
    groupable as a view) the GEMM writes alpha * result + beta * out."""
    lhs, outs = spec.replace(" ", "").split("->")
    a, b = lhs.split(",")
    size = {c: A.shape[a.index(c) + (1 if za else 0)] for c in a}
    size.update({c: B.shape[b.index(c) + (1 if zb else 0)] for c in b})
    bt = [c for c in outs if c in a and c in b]
    mi = [c for c in outs if c in a and c not in b]
    ni = [c for c in outs if c in b and c not in a]
    ki = [c for c in a if c in b and c not in outs]
    if any(c not in outs and c not in ki for c in a + b):
        raise ValueError(f"einsum_rep: an index summed over one operand only in {spec!r}")
    prod = lambda idx: math.prod(size[c] for c in idx)  # noqa: E731
    nb, M, N, K = prod(bt), prod(mi), prod(ni), prod(ki)
    pa = [a.index(c) for c in bt + mi + ki]
    pb = [b.index(c) for c in bt + ki + ni]
    Ap = _as4(A.permute([0] + [1 + p for p in pa]), (R, nb, M, K)) if za else \
        D._as3(A.permute(pa), (nb, M, K)).unsqueeze(0)
    Bp = _as4(B.permute([0] + [1 + p for p in pb]), (R, nb, K, N)) if zb else \
        D._as3(B.permute(pb), (nb, K, N)).unsqueeze(0)
    order = bt + mi + ni
    if out is not None:
        C = out.permute([0] + [1 + outs.index(c) for c in order]).view(R, nb, M, N)
    else:
        C = torch.empty(R, nb, M, N, dtype=torch.float64, device=A.device)
        alpha, beta = 1.0, 0.0
    gemm(Ap, Bp, C, alpha, beta)
    if out is not None:
        return out
    return C.view([R] + [size[c] for c in order]).permute([0] + [1 + order.index(c) for c in outs])


class FusedReplicaBatch:
    """R replicas of one system, one launch per kernel for all of them.

    ``precision`` "fp64", "df64" or "split" (the integrals of
    fricc_gb300.cholesky.split_eris; every sparse term a dense split-BF16x3
    GEMM on the tensor cores, as FRICCSDGPU(precision="split") runs it with
    its defaults); systematic FRI with every contraction class compressed
    (the configuration of the batched-replica workload); replica r draws
    from GlibcRand(seeds[r]), in the reference's order (the T2-term
    compression first, then the W-intermediate one)."""

    def __init__(self, eris: D.DeviceERIs, settings: dict, seeds, precision: str = "df64", level_shift: float = 0.0,
                 graph: bool = False):
        s = {"compression": "fri", "sampling_method": "systematic", "compressed_contractions": ALL_TERMS,
             "unbiased": False}
        s.update(settings)
        if s["compression"] != "fri" or s["sampling_method"] != "systematic" or s.get("unbiased", False) or \
                sorted(s["compressed_contractions"]) != sorted(ALL_TERMS):
            raise ValueError("FusedReplicaBatch runs systematic FRI with every contraction class compressed")
        if precision not in ("fp64", "df64", "split"):
            raise ValueError("FusedReplicaBatch: precision 'fp64', 'df64' or 'split'")
        self.split = precision == "split"
        if self.split and getattr(eris, "vvvv_rebuild", None) is None:
            raise ValueError("precision 'split' needs the integrals of fricc_gb300.cholesky.split_eris")
        if not self.split and eris.vvvvT is None:
            raise ValueError("FusedReplicaBatch needs the FP64 (vv|vv) block (or precision 'split')")
        from .batch import mp2_device
        self.E = eris
        self.precision = precision
        self.df = precision == "df64"
        if self.df:
            eris.prepare_splits()
        if self.split:
            from .cholesky import dense_spmm_ok
            o_, v_ = eris.nocc, eris.mo_energy.numel() - eris.nocc
            ovv, ov = o_ * v_ * v_, o_ * v_
            dims = (o_, o_, v_, v_)
            terms = [(0, 1, 2, 3, o_ * o_), (3, 0, 1, 2, ov), (2, 0, 1, 3, ov), (2, 3, 0, 1, o_ * o_),
                     (0, 1, 2, 3, v_ * v_), (0, 1, 2, 3, 2 * ov), (1, 3, 0, 2, ov), (1, 2, 0, 3, ov)]
            if not all(dense_spmm_ok(dims, *t) for t in terms):
                raise ValueError("FusedReplicaBatch 'split': a sparse term of this size is too small for the "
                                 "tensor cores (run FRICCSDGPU or ReplicaBatch)")
            eris.prepare_tc({"ovvv_iabc": ("A", ovv, v_), "ovvv": ("A", ovv, v_), "ovvv_kacd": ("A", ovv, v_),
                             "g_klcd": ("A", o_, ovv), "g_kldc": ("B", o_ * o_ * v_, v_),
                             "G_t1": ("B", ovv, v_)})
            self._tc_status = torch.zeros(1, dtype=torch.int32, device=eris.device)
            self._vvvv_bt = None
        self.seeds = list(seeds)
        self.R = R = len(self.seeds)
        self.rng = [GlibcRand(sd) for sd in self.seeds]
        self.m = int(s["m_keep"])
        t1, t2 = mp2_device(eris)
        self.o, self.v = t1.shape
        if self.m <= 0 or self.m > t2.numel():
            raise ValueError("Bad m_keep value! The following condition wasn't met 0 < m_keep <= t2.size")
        self.t1 = t1.unsqueeze(0).repeat(R, 1, 1).contiguous()
        self.t2 = t2.unsqueeze(0).repeat(R, 1, 1, 1, 1).contiguous()
        self.lib = L.load()
        self.spb = ctypes.c_void_p()
        st = L.cur_stream()
        L.check(self.lib.fricc_spb_create(R, L.i64arr(t2.shape), self.m, st, ctypes.byref(self.spb)))
        dev = eris.device
        self.rn_dev = torch.zeros(R, 2, dtype=torch.float64, device=dev)
        self.res = torch.zeros(R, 4, dtype=torch.float64, device=dev)
        self._side_owner = L.OwnStream(dev)
        # graph=True: the first step runs eagerly (it makes the compressed
        # handles' bucketings and the first-use operand splits), the second
        # is captured into one CUDA graph that every later step replays
        self.graph = bool(graph)
        self._g = None
        self._cap_owner = None
        self._steps = 0
        self.history = [[] for _ in range(R)]
        o, v = self.o, self.v
        e_o = eris.mo_energy[:o].contiguous()
        e_v = (eris.mo_energy[o:] + float(level_shift)).contiguous()
        self.C = {"foo": eris.fock[:o, :o].contiguous(), "fvv": eris.fock[o:, o:].contiguous(),
                  "fov": eris.fock[:o, o:].contiguous(), "e_o": e_o, "e_v": e_v,
                  "eia": (e_o[:, None] - e_v[None, :]).contiguous()}
        torch.cuda.current_stream().synchronize()

    def __del__(self):
        if getattr(self, "spb", None) is not None and self.spb.value and L._lib is not None:
            L._lib.fricc_spb_destroy(self.spb)
            self.spb = None

    # ------------------------------------------------------------------
    def _mm(self, A, B, C, alpha=1.0, beta=0.0, const=None, const_b=None):
        """The precision's GEMM for every replica; ``const`` / ``const_b``
        name a constant integral operand whose tensor-core split is kept."""
        if self.split:
            from .cholesky import gemm_tc_rep
            E = self.E
            return gemm_tc_rep(A, B, C, alpha, beta, self.R, status=self._tc_status,
                               a_split=E.tc(const, "A") if const else None,
                               b_split=E.tc(const_b, "B") if const_b else None)
        return (D.gemm_df if self.df else D.gemm_f64)(A, B, C, alpha, beta)

    def _spmm(self, which, pa, pb, ka, kb, coef, W, QS, Op, st, const=None):
        """A sparse term of every replica: W shared (``const`` names a
        constant integral block) or stacked [R, ...]; Op stacked."""
        R = self.R
        o_stride = Op[0].numel()
        if self.split:
            from .cholesky import dense_spmm_rep, split_b_rep
            if const is not None:
                Bt, b_rep = self.E.tc_w(const, QS), 0
            else:
                Bt, b_rep = split_b_rep(W, R, QS), QS
            done = dense_spmm_rep(self.spb, which, R, tuple(self.t2.shape[1:]), pa, pb, ka, kb, coef, Bt, b_rep, QS,
                                  Op, self._tc_status)
            assert done, "checked at construction"
        elif self.df:
            if const is not None:
                W2, w_stride = self.E.split(const), 0
            else:
                rows = W[0].numel() // QS
                W2, w_stride = D.split_f2(W.reshape(R * rows, QS), QS), rows * ((QS + 1) // 2)
            L.check(self.lib.fricc_spb_spmm_f2(self.spb, which, pa, pb, ka, kb, float(coef), _ptr(W2), w_stride,
                                               int(QS), _ptr(Op), o_stride, st))
        else:
            w_stride = 0 if const is not None else W[0].numel()
            L.check(self.lib.fricc_spb_spmm(self.spb, which, pa, pb, ka, kb, float(coef), _ptr(W), w_stride,
                                            int(QS), _ptr(Op), o_stride, st))

    def _symadd(self, out, X, coef):
        L.check(self.lib.fricc_symadd_b(_ptr(out), _ptr(X), self.R, self.o, self.v, L.i64arr(X.stride()),
                                        float(coef), L.cur_stream()))

    def _capture(self):
        """One batch step as a CUDA graph on a capture stream of this batch's
        own: it reads the draws from ``rn_dev`` and the amplitudes from
        ``t1``/``t2``, and copies the new amplitudes back into them, so each
        replay advances every replica by one iteration."""
        from .friccsd import _CAPTURE_LOCK
        cur = torch.cuda.current_stream()
        if self._cap_owner is None:
            self._cap_owner = L.OwnStream(self.E.device)
        cap = self._cap_owner.stream
        g = torch.cuda.CUDAGraph()
        with _CAPTURE_LOCK:
            cap.wait_stream(cur)
            with torch.cuda.stream(cap):
                g.capture_begin(capture_error_mode="thread_local")
                try:
                    t1n, t2n = self._update(self.t1, self.t2)
                    self.t1.copy_(t1n)
                    self.t2.copy_(t2n)
                    del t1n, t2n
                finally:
                    g.capture_end()
            cur.wait_stream(cap)
        self._g = g

    def step(self, record: bool = True):
        """One iteration of every replica (with ``graph``, a replay of the
        captured batch step from the second step on)."""
        rn = [[g(), g()] for g in self.rng]
        self.rn_dev.copy_(torch.tensor(rn, dtype=torch.float64))
        if self.graph and self._steps > 0:
            if self._g is None:
                self._capture()
            self._g.replay()
        else:
            self.t1, self.t2 = self._update(self.t1, self.t2)
        self._steps += 1
        r = self.res[:, :2].cpu()
        rep = ctypes.c_int(-1)
        rc = self.lib.fricc_spb_status(self.spb, ctypes.byref(rep))
        if rc:
            L.check(rc)
        if self.split:
            self.E.vvvv_rebuild.check()
            if int(self._tc_status.item()):
                raise L.FriccError(5, "split-precision GEMM: a bounded tensor-core pipeline wait gave up")
        if record:
            for k in range(self.R):
                self.history[k].append(float(r[k, 0]))
        return r.numpy()

    def energies(self) -> np.ndarray:
        return np.array([h[-1] for h in self.history])

    def stats(self):
        e = self.energies()
        return float(e.mean()), float(e.var(ddof=1)) if e.size > 1 else 0.0

    def trace_stats(self, burn: int = 0):
        """Per replica: the mean of its E_corr trace after ``burn``
        iterations, its error bar and its autocorrelation time, as
        fri-cc's mcmc_std gives them (fricc/__init__.py:8-11)."""
        from .batch import ReplicaBatch
        return ReplicaBatch.trace_stats(self, burn)

    def export(self, which: int, r: int):
        """Replica r's entries of compression ``which`` (0: the T2 terms',
        1: the W intermediates') of the last step, as host arrays."""
        flat = np.empty(self.m, dtype=np.int64)
        vals = np.empty(self.m, dtype=np.float64)
        L.check(self.lib.fricc_spb_export(self.spb, int(which), int(r), ctypes.c_void_p(flat.ctypes.data),
                                          ctypes.c_void_p(vals.ctypes.data),
                                          L.cur_stream()))
        return flat, vals

    def _update(self, t1, t2):
        E, R, o, v = self.E, self.R, self.o, self.v
        ov, ovv, oov = o * v, o * v * v, o * o * v
        f64, dev = t2.dtype, t2.device
        comb, mmf, mm = D.combine, D.gemm_f64, self._mm
        C = self.C
        fov = C["fov"]

        def new(*shape):
            return torch.empty(*shape, dtype=f64, device=dev)

        def ein(spec, A_, B_, za, zb, out=None, alpha=1.0, beta=0.0):
            return einsum_rep(spec, A_, B_, mm, za, zb, R, out=out, alpha=alpha, beta=beta)

        main, side = torch.cuda.current_stream(), self._side_owner.stream
        st = ctypes.c_void_p(main.cuda_stream)
        side.wait_stream(main)
        with torch.cuda.stream(side):   # both compressions of every replica, overlapping the dense work
            L.check(self.lib.fricc_spb_recompress_pair(self.spb, _ptr(t2), _ptr(self.rn_dev),
                                                       ctypes.c_void_p(side.cuda_stream)))

        tt, ttp = new(R, o, o, v, v), new(R, v, o, o, v)
        comb([tt, ttp.permute(0, 2, 3, 1, 4)], [t2], [[1.0, 1.0], [1.0, 1.0]],
             prod=[t1[:, :, None, :, None], t1[:, None, :, None, :]])
        Foo0 = new(R, o, o)
        comb([Foo0], [C["foo"]])
        mm(E.g_klcd.view(o, ovv), tt.view(R, o, ovv).transpose(1, 2), Foo0, 1.0, 1.0, const="g_klcd")
        Fvv0 = new(R, v, v)
        comb([Fvv0], [C["fvv"]])
        mm(ttp.view(R, v, oov), E.g_kldc.view(oov, v), Fvv0, -1.0, 1.0, const_b="g_kldc")
        del tt, ttp
        Fov = new(R, o, v)
        comb([Fov], [fov])
        mmf(E.g_ovov.view(ov, ov), t1.reshape(R, ov, 1), Fov.view(R, ov, 1), 1.0, 1.0)
        Foo, Fvv = new(R, o, o), new(R, v, v)
        comb([Foo], [Foo0])
        comb([Foo.diagonal(dim1=1, dim2=2)], [C["e_o"]], [[-1.0]], accumulate=True)
        comb([Fvv], [Fvv0])
        comb([Fvv.diagonal(dim1=1, dim2=2)], [C["e_v"]], [[-1.0]], accumulate=True)

        # T1 equation (fricc/friccsd.py:153-176)
        t1new = new(R, o, v)
        A_ik = new(R, o, o)
        mmf(t1, fov.T, A_ik)
        mmf(A_ik, t1, t1new, -2.0, 0.0)
        mmf(t1, Fvv.transpose(1, 2), t1new, 1.0, 1.0)
        mmf(Foo.transpose(1, 2), t1, t1new, -1.0, 1.0)
        U = new(R, o, v, o, v)
        comb([U], [t2.permute(0, 1, 3, 2, 4), t2.permute(0, 2, 3, 1, 4)], [[2.0, -1.0]])
        mmf(Fov.reshape(R, 1, ov), U.view(R, ov, ov), t1new.view(R, 1, ov), 1.0, 1.0)
        del U
        B_ik = new(R, o, o)
        mmf(t1, Fov.transpose(1, 2), B_ik)
        mmf(B_ik, t1, t1new, 1.0, 1.0)
        comb([t1new], [fov], accumulate=True)
        mmf(t1.reshape(R, 1, ov), E.G_t1_kcia.view(ov, ov), t1new.view(R, 1, ov), 1.0, 1.0)
        mm(t2.view(R, o, ovv), E.G_t1.view(ovv, v), t1new, 1.0, 1.0, const_b="G_t1")
        X = new(R, v, v)
        mmf(t1.reshape(R, 1, ov), E.G_t1_kdca.view(ov, v * v), X.view(R, 1, v * v))
        mmf(t1, X, t1new, 1.0, 1.0)
        ein("lcki,klac->ia", E.g_ovoo, t2, False, True, out=t1new, alpha=-1.0, beta=1.0)
        u_ki = new(R, o, o)
        mmf(t1.reshape(R, 1, ov), E.g_ovoo.view(ov, o * o), u_ki.view(R, 1, o * o))
        mmf(u_ki.transpose(1, 2), t1, t1new, -1.0, 1.0)

        # T2 driver terms (:179-187)
        Y1 = ein("kibc,jc->kibj", E.oovv, t1, False, True)
        Rr = new(R, ovv, o)
        mm(E.ovvv_iabc.view(ovv, v), t1.transpose(1, 2), Rr, 1.0, 0.0, const="ovvv_iabc")
        tmp = new(R, o, o, v, v)
        comb([tmp], [Rr.view(R, o, v, v, o).permute(0, 1, 4, 2, 3), ein("ka,kibj->ijab", t1, Y1, True, True)],
             [[1.0, -1.0]])
        del Y1
        t2new = new(R, o, o, v, v)
        comb([t2new], [E.ovov.permute(0, 2, 1, 3)])
        self._symadd(t2new, tmp, 1.0)
        tmp2 = new(R, v, o, o, o)
        comb([tmp2], [ein("kcai,jc->akij", E.ovvo, t1, False, True), E.ovoo.permute(1, 3, 0, 2)])
        self._symadd(t2new, ein("akij,kb->ijab", tmp2, t1, True, True), -1.0)
        del tmp, tmp2

        Loo = new(R, o, o)
        comb([Loo], [Foo0])
        mmf(fov, t1.transpose(1, 2), Loo, 1.0, 1.0)
        comb([Loo], [u_ki], accumulate=True)
        Lvv = new(R, v, v)
        comb([Lvv], [Fvv0])
        mmf(t1.transpose(1, 2), fov, Lvv, -1.0, 1.0)
        comb([Lvv], [X.transpose(1, 2)], accumulate=True)
        comb([Loo.diagonal(dim1=1, dim2=2)], [C["e_o"]], [[-1.0]], accumulate=True)
        comb([Lvv.diagonal(dim1=1, dim2=2)], [C["e_v"]], [[-1.0]], accumulate=True)

        main.wait_stream(side)  # the compressed tensors from here on
        # sparse_cc_Woooo (:309-322)
        Wo = new(R, o, o, o, o)                                                   # [i,j,k,l]
        comb([Wo.permute(0, 3, 4, 1, 2)], [ein("lcki,jc->klij", E.ovoo, t1, False, True),
                                           ein("kclj,ic->klij", E.ovoo, t1, False, True)])
        self._spmm(1, 0, 1, 2, 3, 1.0, E.ovov_cdkl, o * o, Wo, st, const="ovov_cdkl")        # 1323
        Woooo = Wo.permute(0, 3, 4, 1, 2)                                         # (k,l,i,j)
        comb([Woooo], [ein("kild,jd->klij", ein("kcld,ic->kild", E.ovov, t1, False, True), t1, True, True)],
             accumulate=True)
        comb([Woooo], [E.oooo.permute(0, 2, 1, 3)], accumulate=True)

        # sparse_cc_Wvoov / sparse_cc_Wvovo (:334-376)
        Rr = new(R, ovv, o)
        mm(E.ovvv.view(ovv, v), t1.transpose(1, 2), Rr, 1.0, 0.0, const="ovvv")
        Wp = new(R, v, o, o, v)                                                   # [a,i,k,c]
        Wvoov = Wp.permute(0, 1, 3, 2, 4)                                         # (a,k,i,c)
        comb([Wvoov], [Rr.view(R, o, v, v, o).permute(0, 3, 1, 4, 2), ein("kcli,la->akic", E.ovoo, t1, False, True),
                       E.ovvo.permute(2, 0, 3, 1)], [[1.0, -1.0, 1.0]])
        self._spmm(1, 3, 0, 1, 2, -0.5, E.ovov, ov, Wp, st, const="ovov")                        # 0112
        self._spmm(1, 2, 0, 1, 3, 1.0, E.ovov_0313_0113, ov, Wp, st, const="ovov_0313_0113")     # 0313+0113
        comb([Wvoov], [ein("lkci,la->akic", ein("ldkc,id->lkci", E.ovov, t1, False, True), t1, True, True)],
             [[-1.0]], accumulate=True)
        mm(E.ovvv_kacd.view(ovv, v), t1.transpose(1, 2), Rr, 1.0, 0.0, const="ovvv_kacd")
        Wq = new(R, v, o, o, v)                                                   # [a,i,k,c]
        Wvovo = Wq.permute(0, 1, 3, 4, 2)                                         # (a,k,c,i)
        comb([Wvovo], [Rr.view(R, o, v, v, o).permute(0, 2, 1, 3, 4), ein("lcki,la->akci", E.ovoo, t1, False, True),
                       E.oovv.permute(2, 0, 3, 1)], [[1.0, -1.0, 1.0]])
        self._spmm(1, 3, 0, 1, 2, -0.5, E.ovov_0312, ov, Wq, st, const="ovov_0312")              # 0312
        comb([Wvovo], [ein("lkci,la->akci", ein("lckd,id->lkci", E.ovov, t1, False, True), t1, True, True)],
             [[-1.0]], accumulate=True)
        del Rr

        # 0101
        comb([t2new], [ein("lija,lb->ijab", ein("klij,ka->lija", Woooo, t1, True, True), t1, True, True)],
             accumulate=True)
        Tp = new(R, v, v, o, o)                                                   # [a,b,i,j]
        comb([Tp], [t2new.permute(0, 3, 4, 1, 2)])
        Wk = new(R, o, o, o, o)
        comb([Wk], [Woooo])
        self._spmm(0, 2, 3, 0, 1, 1.0, Wk, o * o, Tp, st)
        comb([t2new], [Tp.permute(0, 3, 4, 1, 2)])
        del Tp, Wk

        # Wvvvv terms (:207, :222-234); fricc/friccsd.py:222 sums c,d inside Wvvvv
        S = new(R, v, v)
        comb([S], [E.S0])
        mmf(E.U.T, t1, S, -1.0, 1.0)
        mmf(t1.transpose(1, 2), E.U, S, -1.0, 1.0)
        comb([t2new], [], [[1.0]], prod=[S[:, None, None, :, :], t1[:, :, None, :, None], t1[:, None, :, None, :]],
             accumulate=True)
        if self.split:   # (ac|bd) rebuilt from the split factor straight into the B operand
            from .cholesky import dense_spmm_rep
            self._vvvv_bt = E.vvvv_rebuild.rebuild_split_b(self._vvvv_bt)
            dense_spmm_rep(self.spb, 0, R, (o, o, v, v), 0, 1, 2, 3, 1.0, self._vvvv_bt, 0, v * v, t2new,
                           self._tc_status)                                       # 2323
        else:
            self._spmm(0, 0, 1, 2, 3, 1.0, E.vvvvT, v * v, t2new, st, const="vvvvT")             # 2323
        XY = D.zero(new(R, o, o, 2, o, v))
        self._spmm(0, 0, 1, 2, 3, 1.0, E.ovvv_XY, 2 * ov, XY, st, const="ovvv_XY")           # t1 parts
        XYv = XY.view(R, o * o, 2, o, v)
        t2v = t2new.view(R, o * o, v, v)
        mm(XYv[:, :, 0].transpose(2, 3), t1.unsqueeze(1).expand(R, o * o, o, v), t2v, -1.0, 1.0)
        mm(t1.transpose(1, 2).unsqueeze(1).expand(R, o * o, v, o), XYv[:, :, 1], t2v, -1.0, 1.0)
        del XY

        tmpL = new(R, o, o, v, v)
        mm(Lvv.unsqueeze(1).expand(R, o * o, v, v), t2.view(R, o * o, v, v), tmpL.view(R, o * o, v, v), 1.0, 0.0)
        self._symadd(t2new, tmpL, 1.0)                                            # Lvv t2, :238-239
        mm(Loo.transpose(1, 2), t2.view(R, o, ovv), tmpL.view(R, o, ovv), 1.0, 0.0)
        self._symadd(t2new, tmpL, -1.0)                                           # Loo t2, :240-241
        del tmpL

        WA, WB, W2 = new(R, o, v, o, v), new(R, o, v, o, v), new(R, o, v, o, v)  # [k,c,i,a]
        comb([WA, WB, W2], [Wvoov.permute(0, 2, 4, 3, 1), Wvovo.permute(0, 2, 3, 4, 1)],
             [[1.0, 0.0], [0.0, 1.0], [2.0, -1.0]])
        tmp = D.zero(new(R, o, v, o, v))                                          # [j,b,i,a]
        self._spmm(0, 1, 3, 0, 2, 1.0, W2, ov, tmp, st)                           # 1302 + 1202
        self._symadd(t2new, tmp.permute(0, 3, 1, 4, 2), 1.0)
        D.zero(tmp)
        self._spmm(0, 1, 2, 0, 3, 1.0, WA, ov, tmp, st)                           # 1303
        self._symadd(t2new, tmp.permute(0, 3, 1, 4, 2), -1.0)
        D.zero(tmp)
        self._spmm(0, 1, 2, 0, 3, 1.0, WB, ov, tmp, st)                           # 1203, [j,a,i,b]
        self._symadd(t2new, tmp.permute(0, 3, 1, 2, 4), -1.0)
        del WA, WB, W2, tmp

        # denominators + energy + step norm (:281-284, :418-427)
        L.check(self.lib.fricc_energy_update_batch(R, _ptr(t1new), _ptr(t2new), _ptr(C["eia"]), _ptr(fov),
                                                   _ptr(E.ovov), _ptr(t1), _ptr(t2), o, v, _ptr(t1new), _ptr(t2new),
                                                   _ptr(self.res), st))
        return t1new, t2new
