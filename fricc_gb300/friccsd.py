"""GPU FRI-CCSD: the amplitude iteration of fri-cc's fricc/friccsd.py on GB300.

``FRICCSDGPU`` keeps the integrals, the amplitudes and the two compressed
T2 handles resident in HBM and runs ``update_amps`` (fricc/friccsd.py:29-301)
and ``kernel`` (:379-456) on the device:

* both FRI compressions per iteration (:100-117) on the CUDA library, bit
  for bit the reference's, with the reference's draws (libc ``rand()`` by
  default, in the reference's order: the T2-term compression first, then the
  W-intermediate one);
* the eleven compressed terms (:214, :227, :247-267, :316, :348-356, :372)
  through ``fricc_contract``;
* the denominators, the CCSD energy and the step norm fused in
  ``fricc_energy_update``;
* the dense remainder (Fock-like intermediates, the T1 equation, the dense
  W builds) as GEMMs of the library: FP64 DFMA (``fricc_gemm_f64``), FP32
  pairs (df64) or split-BF16x3 on the tensor cores (split).

Settings are the reference's ``fri_settings`` keys.  The reference reads
``fri_settings["unbiased"]`` (:109), a key its defaults never set (they set
"unbias"); a missing key is treated as False here.  With "unbiased" true,
the W-intermediate compression takes, after ``burn_in`` iterations, the
running average of the T2 inputs (:108-136, the formula as written, FP64
and bit for bit); the iteration counter the reference reads there
(``cc._iter``) is never defined by it, and is here the number of
``update_amps`` calls this solver has run (``reset_average()`` zeroes it).

``update_amps_host`` is the end-to-end entry: host (numpy) amplitudes in,
host amplitudes out, the copies included.
"""
from __future__ import annotations

import ctypes
import threading
import time

import numpy as np
import torch

from . import _lib as L
from . import rccsd_dense as D
from .py_rccsd import libc_uniform

ALLOWED_CONTRACTIONS = ("O^2V^4", "O^3V^3", "O^4V^2")
_CAPTURE_LOCK = threading.Lock()
DEFAULT_SETTINGS = {
    "m_keep": 1000,
    "compression": "fri",
    "sampling_method": "systematic",
    "verbose": False,
    "compressed_contractions": ["O^2V^4", "O^3V^3", "O^4V^2"],
    "burn_in": 100,
    "unbias": False,
}


def _ptr(t: torch.Tensor) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr())


def _sym(x):
    return x + x.permute(1, 0, 3, 2)


def _check_sampling(s, rn_draw):
    if s["compression"] != "fri":
        return
    if s["sampling_method"] not in ("systematic", "pivotal"):
        raise ValueError(f"sampling_method must be 'pivotal' or 'systematic', got {s['sampling_method']!r}")
    if s["sampling_method"] == "pivotal" and not (rn_draw is libc_uniform or hasattr(rn_draw, "history")):
        raise ValueError("pivotal sampling draws from the process's rand() (rn_draw=libc_uniform) or from a "
                         "GlibcRand stream; a generic draw callable cannot supply them")


def _compress(handle, t2, m, s, rn, rn_draw, stream):
    """One compression as the settings ask: systematic/largest take the draw rn,
    pivotal draws its own from rn_draw."""
    if s["compression"] == "fri" and s["sampling_method"] == "pivotal":
        return handle.compress_pivotal(t2, m, None if rn_draw is libc_uniform else rn_draw, stream)
    return handle.compress(t2, m, s["compression"], rn, stream)


class _Handle:
    """A reusable compressed-T2 handle (device SparseTensor4d)."""

    def __init__(self):
        self.h = ctypes.c_void_p()
        self.key = None

    def compress(self, t2, m, compression, rn, stream):
        lib = L.load()
        key = (tuple(t2.shape), int(m))
        comp = L.COMPRESSION[compression]
        if self.h.value and self.key == key:
            L.check(lib.fricc_sp_recompress(self.h, _ptr(t2), comp, 0, float(rn), stream))
        else:
            self.free()
            L.check(lib.fricc_sp_create(_ptr(t2), L.i64arr(t2.shape), int(m), comp, 0, float(rn), stream,
                                        ctypes.byref(self.h)))
            self.key = key
        return self.h

    def compress_dev(self, t2, m, compression, rn_ptr, stream):
        """Re-compress an existing handle with the draw read from device memory
        (rn_ptr): stream-ordered work only, capturable in a CUDA graph."""
        if not self.h.value or self.key != (tuple(t2.shape), int(m)):
            raise RuntimeError("compress_dev needs a handle created for this shape")
        L.check(L.load().fricc_sp_recompress_dev(self.h, _ptr(t2), L.COMPRESSION[compression], 0, rn_ptr, stream))
        return self.h

    def compress_pivotal(self, t2, m, rng, stream):
        """Pivotal FRI compression drawing from rng (GlibcRand: on the device;
        the process's rand() otherwise)."""
        lib = L.load()
        key = (tuple(t2.shape), int(m))
        hist, writeback = L.hist_arg(rng)
        used = ctypes.c_int64(0)
        if self.h.value and self.key == key:
            L.check(lib.fricc_sp_recompress_pivotal(self.h, _ptr(t2), hist, stream, ctypes.byref(used)))
        else:
            self.free()
            L.check(lib.fricc_sp_create_pivotal(_ptr(t2), L.i64arr(t2.shape), int(m), hist, stream,
                                                ctypes.byref(self.h), ctypes.byref(used)))
            self.key = key
        writeback()
        self.draws_used = used.value
        return self.h

    def ready_for(self, t2, m):
        return bool(self.h.value) and self.key == (tuple(t2.shape), int(m))

    def free(self):
        if self.h.value and L._lib is not None:
            L._lib.fricc_sp_destroy(self.h)
        self.h = ctypes.c_void_p()

    def __del__(self):
        self.free()


class FRICCSDGPU:
    def __init__(self, eris: D.DeviceERIs, fri_settings=None, level_shift=0.0, rn_draw=libc_uniform,
                 wvvvv_t1t1="reference", precision="fp64", graph=False, rebuild_vvvv=True, split_sparse="dense",
                 autotune=False):
        s = dict(DEFAULT_SETTINGS)
        s.update(fri_settings or {})
        for c in s["compressed_contractions"]:
            if c not in ALLOWED_CONTRACTIONS:
                raise ValueError(f"Contraction ({c}) is not supported!")
        if s["compression"] not in L.COMPRESSION:
            raise ValueError(f"The compression method you chose ({s['compression']}) isn't supported")
        _check_sampling(s, rn_draw)
        self.settings = s
        self.eris = eris
        self.level_shift = float(level_shift)
        self.rn_draw = rn_draw
        self.wvvvv_t1t1 = wvvvv_t1t1
        if precision not in ("fp64", "df64", "split"):
            raise ValueError("precision must be 'fp64', 'df64' or 'split'")
        if precision == "split":
            if getattr(eris, "vvvv_rebuild", None) is None:
                raise ValueError("precision 'split' needs the integrals of fricc_gb300.cholesky.split_eris")
            if wvvvv_t1t1 != "reference" or "O^2V^4" not in s["compressed_contractions"]:
                raise ValueError("precision 'split' contracts (vv|vv) only through the compressed O^2V^4 term")
        elif eris.vvvvT is None:
            raise ValueError("these integrals keep no FP64 (vv|vv) block: use precision 'split'")
        self.precision = precision
        self._df = precision in ("df64", "split")   # FP32-pair sparse terms and dense GEMMs
        # split precision: rebuild (vv|vv) from the factor every iteration (it
        # is never resident), or once and keep the FP32 block
        self.rebuild_vvvv = bool(rebuild_vvvv)
        # split precision, sparse terms: the compressed T zero-filled into a
        # dense split-BF16x3 GEMM on the tensor cores ("dense"), or the sparse
        # kernels against FP32 W with plain FP32 sums ("fp32", also the
        # fallback for GEMMs too small for the tensor cores) or with T values
        # and sums in float pairs ("pairs")
        if split_sparse not in ("dense", "fp32", "pairs"):
            raise ValueError("split_sparse must be 'dense', 'fp32' or 'pairs'")
        self.split_sparse = split_sparse
        # df64: time the launch configurations of every sparse term and
        # FP32-pair GEMM shape on first use and keep the fastest
        from .autotune import Autotuner
        self._tuner = Autotuner() if (autotune and precision == "df64") else None
        self._spmm32 = L.load().fricc_spmm_f1 if split_sparse == "pairs" else L.load().fricc_spmm_f32
        self._dims = None
        self._vvvv_bt = None
        self._vvvv_buf = None
        self._tc_status = torch.zeros(1, dtype=torch.int32, device=eris.device)
        self.lib = L.load()
        if precision == "df64":
            eris.prepare_splits()
        elif precision == "split":
            o_, v_ = eris.nocc, eris.mo_energy.numel() - eris.nocc
            eris.prepare_f32({"ovvv_XY": 2 * o_ * v_, "ovov": o_ * v_, "ovov_0313_0113": o_ * v_,
                              "ovov_0312": o_ * v_, "ovov_cdkl": o_ * o_})
            ovv = o_ * v_ * v_
            eris.prepare_tc({"ovvv_iabc": ("A", ovv, v_), "ovvv": ("A", ovv, v_), "ovvv_kacd": ("A", ovv, v_),
                             "g_klcd": ("A", o_, ovv), "g_kldc": ("B", o_ * o_ * v_, v_),
                             "G_t1": ("B", ovv, v_)})
        self._sp = _Handle()
        self._sp_w = _Handle()
        # streams of this solver alone (torch's pool hands the same few streams
        # to everyone, which would tie solvers on different threads together)
        self._side_owner = L.OwnStream(eris.device)
        self._side = self._side_owner.stream
        self.graph = bool(graph)
        self._g = None
        self._g_key = None
        self._cap = None
        self._res = torch.zeros(4, dtype=torch.float64, device=eris.device)
        self._wT = None
        self._iter = 0
        self._t2_avg = None
        self.timings = {}
        self.last_energy = None
        self.last_normt = None
        self.launches = 0

    # ------------------------------------------------------------------
    def _contract(self, term, W, T, out, stream):
        L.check(self.lib.fricc_contract(term.encode(), _ptr(W), L.i64arr(W.shape), L.i64arr(W.stride()), T,
                                        _ptr(out), L.i64arr(out.shape), L.i64arr(out.stride()), stream))

    def _spmm(self, T, pa, pb, ka, kb, coef, Wp, QS, Op, stream, const=None):
        """Op[P][q] += coef * sum_e Wp[key_e][q] value_e (both contiguous).

        With precision "df64" the products and sums run in FP32-pair
        arithmetic; ``const`` names a constant integral block whose split
        form is cached on the DeviceERIs."""
        assert Wp.is_contiguous() and Op.is_contiguous()
        if self.precision == "split":
            if self.split_sparse == "dense":
                # the compressed T zero-filled into a split-BF16x3 operand and
                # contracted on the tensor cores
                from .cholesky import dense_spmm, dense_spmm_ok, split_b
                if dense_spmm_ok(self._dims, pa, pb, ka, kb, QS):
                    Bt = self.eris.tc_w(const, QS) if const else split_b(Wp.reshape(-1, QS))
                    dense_spmm(T, self._dims, pa, pb, ka, kb, coef, Bt, QS, Op, self._tc_status)
                    return
            # the integrals carry split-BF16x3 error (~2^-16): W' in FP32
            # (half the bytes of the float-pair layout)
            W32 = self.eris.f32(const, QS) if const else D.to_f32_rows(Wp, QS)
            L.check(self._spmm32(T, pa, pb, ka, kb, float(coef), _ptr(W32), int(QS), W32.shape[1], _ptr(Op), stream))
        elif self._df:
            W2 = self.eris.split(const) if const else D.split_f2(Wp, QS)
            assert W2.numel() == (Wp.numel() // QS) * ((QS + 1) // 2) * 4, "float-pair W' split with another QS"

            def launch(outs):
                L.check(self.lib.fricc_spmm_f2(T, pa, pb, ka, kb, float(coef), _ptr(W2), int(QS), _ptr(outs[0]),
                                               stream))
            if self._tuner is not None:
                from .autotune import SPMM_CANDIDATES
                self._tuner.run(("spmm", pa, pb, ka, kb, int(QS), self._dims), SPMM_CANDIDATES, launch, [Op])
            else:
                launch([Op])
        else:
            L.check(self.lib.fricc_spmm(T, pa, pb, ka, kb, float(coef), _ptr(Wp), int(QS), _ptr(Op), stream))

    def _tuned_compress(self, t2, m, launch):
        """Run a paired compression; with the autotuner, its select-digit
        width is timed over the candidates on first use of the shape (each
        candidate recompresses the same T2 with the same draws, and every
        width keeps the same entries) and the fastest replayed."""
        if self._tuner is None:
            return launch(None)
        from .autotune import COMPRESS_CANDIDATES
        self._tuner.run(("compress_pair", tuple(t2.shape), int(m)), COMPRESS_CANDIDATES, launch, [])

    def update_amps(self, t1, t2, rn=None, t1_old=None, t2_old=None):
        """One iteration on device tensors; returns (t1new, t2new).  With
        ``graph=True`` (and systematic or "largest" compression, no unbiased
        averaging) the iteration after the first is captured once into a CUDA
        graph and replayed: the host work per iteration drops to a few copies
        and one launch, and the results are the same as eager execution."""
        s = self.settings
        if (self.graph and t1_old is None and t2_old is None and not s.get("unbiased", False) and not s["verbose"]
                and not (s["compression"] == "fri" and s["sampling_method"] == "pivotal")
                and self._sp.h.value):
            return self._update_graph(t1, t2, rn)
        return self._update_eager(t1, t2, rn, t1_old, t2_old)

    def _update_graph(self, t1, t2, rn):
        s = self.settings
        comp = s["compressed_contractions"]
        need_w = "O^3V^3" in comp or "O^4V^2" in comp
        if rn is None:
            rn = [self.rn_draw() if s["compression"] == "fri" else 0.0 for _ in range(2 if need_w else 1)]
        key = (tuple(t1.shape), tuple(t2.shape))
        if self._g is None or self._g_key != key:
            dev = t2.device
            self._gs_t1 = t1.contiguous().clone()
            self._gs_t2 = t2.contiguous().clone()
            self._rn_dev = torch.zeros(2, dtype=torch.float64, device=dev)
            # each solver captures on its own stream, without the device-wide
            # synchronisation torch.cuda.graph() performs (other host threads
            # may be replaying or capturing their own solvers meanwhile);
            # captures themselves are serialised
            cur = torch.cuda.current_stream()
            if self._cap is None:
                self._cap_owner = L.OwnStream(dev)
                self._cap = self._cap_owner.stream
            g = torch.cuda.CUDAGraph()
            with _CAPTURE_LOCK:
                self._cap.wait_stream(cur)
                with torch.cuda.stream(self._cap):
                    g.capture_begin(capture_error_mode="thread_local")
                    try:
                        out = self._update_eager(self._gs_t1, self._gs_t2, None, None, None, rn_dev=self._rn_dev)
                    finally:
                        g.capture_end()
                cur.wait_stream(self._cap)
            self._g, self._g_key, self._g_out = g, key, out
        self._rn_dev.copy_(torch.tensor(list(rn) + [0.0] * (2 - len(rn)), dtype=torch.float64))
        if t1.data_ptr() != self._gs_t1.data_ptr():
            self._gs_t1.copy_(t1)
        if t2.data_ptr() != self._gs_t2.data_ptr():
            self._gs_t2.copy_(t2)
        self._g.replay()
        self._iter += 1
        return self._g_out[0].clone(), self._g_out[1].clone()

    def _update_eager(self, t1, t2, rn=None, t1_old=None, t2_old=None, rn_dev=None):
        """One iteration, every kernel launched from the host.

        rn: the two uniform draws (compression #1, #2); default rn_draw().
        After the call, read_energy() gives E_corr(t1new, t2new) and the step
        norm against (t1_old, t2_old) (default: the inputs).

        Same algebra as fricc/friccsd.py:29-301, arranged for the GPU:
        * the O^2V^3 T1 terms are one GEMM against a combined integral;
        * Wvvvv is never materialised: its (ac|bd) part is contracted with the
          compressed T2 directly (the 2323 term) and its two t1 parts become
          two O^3V^3-sized sparse contractions X, Y followed by a t1 GEMM;
        * 1302 and 1202 (and 0313 and 0113) share bucketing and output, so
          each pair runs as one pass over a combined W.
        Each rearrangement changes results only at the level of FP64 rounding.
        """
        self._dims = tuple(t2.shape)
        E = self.eris
        s = self.settings
        m = int(s["m_keep"])
        if m > t2.numel() or m == 0:
            raise ValueError("Bad m_keep value! The following condition wasn't met 0 < m_keep <= t2.size")
        comp = s["compressed_contractions"]
        o, v = t1.shape
        ov = o * v
        st = L.cur_stream()
        t2 = t2.contiguous()
        t1 = t1.contiguous()
        ein = torch.einsum
        need_w = "O^3V^3" in comp or "O^4V^2" in comp
        piv = s["compression"] == "fri" and s["sampling_method"] == "pivotal"
        if rn is None and rn_dev is None:
            kind = s["compression"]
            rn = [self.rn_draw() if kind == "fri" and not piv else 0.0 for _ in range(2 if need_w else 1)]
        # both compressions run on a side stream, overlapping the dense work
        # below; the sparse terms wait for them
        # (t2 needs no record_stream on the side stream: the main stream waits
        # for the side stream below, before anything the caller can free
        # or allocate after this call)
        main, side = torch.cuda.current_stream(), self._side
        side.wait_stream(main)
        with torch.cuda.stream(side):
            sst = ctypes.c_void_p(side.cuda_stream)
            # both compressions of the same T2 (systematic FRI, no running
            # average): one paired pass, bit-identical to two
            ws = t2 if (rn_dev is not None or not need_w) else self._w_source(t2)  # once: it may update
            verbose = bool(s["verbose"]) and rn_dev is None   # one phase table per compression, as the reference
            paired = (need_w and s["compression"] == "fri" and s["sampling_method"] == "systematic"
                      and self._sp.ready_for(t2, m) and self._sp_w.ready_for(t2, m) and ws is t2 and not verbose)
            if paired and rn_dev is not None:  # captured: draws from device memory
                self._tuned_compress(t2, m, lambda _: L.check(self.lib.fricc_sp_recompress_pair_dev(
                    self._sp.h, self._sp_w.h, _ptr(t2), ctypes.c_void_p(rn_dev.data_ptr()), sst)))
                T, Tw = self._sp.h, self._sp_w.h
            elif paired:
                self._tuned_compress(t2, m, lambda _: L.check(self.lib.fricc_sp_recompress_pair(
                    self._sp.h, self._sp_w.h, _ptr(t2), float(rn[0]), float(rn[1]), sst)))
                T, Tw = self._sp.h, self._sp_w.h
            elif rn_dev is not None:  # captured: draws from device memory, handles exist
                T = self._sp.compress_dev(t2, m, s["compression"], ctypes.c_void_p(rn_dev.data_ptr()), sst)
                Tw = self._sp_w.compress_dev(t2, m, s["compression"], ctypes.c_void_p(rn_dev.data_ptr() + 8),
                                             sst) if need_w else None
            else:
                T = self._timed(verbose, lambda: _compress(self._sp, t2, m, s, rn[0], self.rn_draw, sst))
                Tw = self._timed(verbose, lambda: _compress(self._sp_w, ws, m, s, rn[1], self.rn_draw, sst)) \
                    if need_w else None
        if rn_dev is None:
            self._iter += 1

        if self.precision == "split":   # split-BF16x3 on the tensor cores (FP32-pair where the grid is too small)
            from .cholesky import gemm_tc
            tcs = self._tc_status

            def mm(A_, B_, C_, alpha=1.0, beta=0.0, const=None, const_b=None):
                return gemm_tc(A_, B_, C_, alpha, beta, status=tcs,
                               a_split=E.tc(const, "A") if const else None,
                               b_split=E.tc(const_b, "B") if const_b else None)

        else:
            mm0 = D.gemm_df if self._df else D.gemm_f64
            tuner = self._tuner

            def mm(A_, B_, C_, alpha=1.0, beta=0.0, const=None, const_b=None):
                if tuner is None:
                    return mm0(A_, B_, C_, alpha, beta)
                from .autotune import GEMM_CANDIDATES
                key = ("gemm", tuple(A_.shape), A_.stride(), tuple(B_.shape), B_.stride(), tuple(C_.shape),
                       C_.stride(), beta != 0.0)
                tuner.run(key, GEMM_CANDIDATES, lambda outs: mm0(A_, B_, outs[0], alpha, beta), [C_])
                return C_

        f64, dev = t2.dtype, t2.device
        comb, mmf = D.combine, D.gemm_f64   # elementwise passes; small GEMMs and GEMVs, FP64 in every form
        C = self._constants(o, v)
        fov, e_o, e_v = C["fov"], C["e_o"], C["e_v"]

        def new(*shape):
            return torch.empty(*shape, dtype=f64, device=dev)

        def ein2(spec, A_, B_, out=None, alpha=1.0, beta=0.0):   # two-operand contractions on mm
            return D.einsum_df(spec, A_, B_, gemm=mm, out=out, alpha=alpha, beta=beta)

        # cc_Foo / cc_Fvv share tt[p,q,r,s] = t2 + t1[p,r] t1[q,s]; cc_Fvv reads it as [r,p,q,s]
        tt, ttp = new(o, o, v, v), new(v, o, o, v)
        comb([tt, ttp.permute(1, 2, 0, 3)], [t2], [[1.0, 1.0], [1.0, 1.0]],
             prod=[t1[:, None, :, None], t1[None, :, None, :]])
        Foo0 = new(o, o)                                   # f_ki + sum_lcd g[k,c,l,d] tt[i,l,c,d]
        comb([Foo0], [C["foo"]])
        mm(E.g_klcd.view(o, o * v * v), tt.view(o, o * v * v).T, Foo0, 1.0, 1.0, const="g_klcd")
        Fvv0 = new(v, v)                                   # f_ac - sum_kld g[k,c,l,d] tt[k,l,a,d]
        comb([Fvv0], [C["fvv"]])
        mm(ttp.view(v, o * o * v), E.g_kldc.view(o * o * v, v), Fvv0, -1.0, 1.0, const_b="g_kldc")
        del tt, ttp
        Fov = new(o, v)                                    # cc_Fov: f_kc + sum_ld g[k,c,l,d] t_ld
        comb([Fov], [fov])
        mmf(E.g_ovov.view(ov, ov), t1.reshape(ov, 1), Fov.view(ov, 1), 1.0, 1.0)
        Foo, Fvv = new(o, o), new(v, v)
        comb([Foo], [Foo0])
        comb([Foo.diagonal()], [e_o], [[-1.0]], accumulate=True)
        comb([Fvv], [Fvv0])
        comb([Fvv.diagonal()], [e_v], [[-1.0]], accumulate=True)

        # T1 equation (fricc/friccsd.py:153-176)
        t1new = new(o, v)
        A_ik = new(o, o)
        mmf(t1, fov.T, A_ik)                               # A[i,k] = sum_c t_ic f_kc
        mmf(A_ik, t1, t1new, -2.0, 0.0)                    # -2 sum_kc f_kc t_ka t_ic
        mmf(t1, Fvv.T, t1new, 1.0, 1.0)                    # + sum_c Fvv[a,c] t_ic
        mmf(Foo.T, t1, t1new, -1.0, 1.0)                   # - sum_k Foo[k,i] t_ka
        U = new(o, v, o, v)                                # U[k,c,i,a] = 2 t2[k,i,c,a] - t2[i,k,c,a]
        comb([U], [t2.permute(0, 2, 1, 3), t2.permute(1, 2, 0, 3)], [[2.0, -1.0]])
        mmf(Fov.reshape(1, ov), U.view(ov, ov), t1new.view(1, ov), 1.0, 1.0)   # 2 Fov t2 - Fov t2
        del U
        B_ik = new(o, o)
        mmf(t1, Fov.T, B_ik)                               # B[i,k] = sum_c t_ic Fov_kc
        mmf(B_ik, t1, t1new, 1.0, 1.0)                     # + sum_kc Fov_kc t_ic t_ka
        comb([t1new], [fov], accumulate=True)              # + f_ia
        mmf(t1.reshape(1, ov), E.G_t1_kcia.view(ov, ov), t1new.view(1, ov), 1.0, 1.0)  # 2 (kc|ai) t - (ki|ac) t
        mm(t2.view(o, o * v * v), E.G_t1.view(o * v * v, v), t1new, 1.0, 1.0, const_b="G_t1")  # O^2V^3, :165-166
        # X[c,a] = sum_kd t1[k,d] (2 (kd|ac) - (kc|ad)): the t1.t1 T1 term (:167-168) and Lvv's ovvv part
        X = new(v, v)
        mmf(t1.reshape(1, ov), E.G_t1_kdca.view(ov, v * v), X.view(1, v * v))
        mmf(t1, X, t1new, 1.0, 1.0)
        # -2 (lc|ki) + (kc|li) = -g_ovoo[l,c,k,i]
        ein2("lcki,klac->ia", E.g_ovoo, t2, out=t1new, alpha=-1.0, beta=1.0)
        u_ki = new(o, o)                                   # u[k,i] = sum_lc t_lc g_ovoo[l,c,k,i]
        mmf(t1.reshape(1, ov), E.g_ovoo.view(ov, o * o), u_ki.view(1, o * o))
        mmf(u_ki.T, t1, t1new, -1.0, 1.0)                  # - sum_k u[k,i] t_ka

        # T2 driver terms (:179-187)
        Y1 = ein2("kibc,jc->kibj", E.oovv, t1)
        R = new(o * v * v, o)                              # R[(i,a,b), j] = sum_c (ia|cb) t_jc
        mm(E.ovvv_iabc.view(o * v * v, v), t1.T, R, 1.0, 0.0, const="ovvv_iabc")
        tmp = new(o, o, v, v)
        comb([tmp], [R.view(o, v, v, o).permute(0, 3, 1, 2), ein2("ka,kibj->ijab", t1, Y1)], [[1.0, -1.0]])
        del Y1
        t2new = new(o, o, v, v)
        comb([t2new], [E.ovov.permute(0, 2, 1, 3)])
        D.sym_add(t2new, tmp, 1.0)
        tmp2 = new(v, o, o, o)
        comb([tmp2], [ein2("kcai,jc->akij", E.ovvo, t1), E.ovoo.permute(1, 3, 0, 2)])
        D.sym_add(t2new, ein2("akij,kb->ijab", tmp2, t1), -1.0)
        del tmp, tmp2

        Loo = new(o, o)                                    # Loo = cc_Foo + f t1^T + sum_lc t_lc g_ovoo[l,c,k,i]
        comb([Loo], [Foo0])
        mmf(fov, t1.T, Loo, 1.0, 1.0)
        comb([Loo], [u_ki], accumulate=True)
        Lvv = new(v, v)                                    # Lvv with its ovvv part from X
        comb([Lvv], [Fvv0])
        mmf(t1.T, fov, Lvv, -1.0, 1.0)
        comb([Lvv], [X.T], accumulate=True)
        comb([Loo.diagonal()], [e_o], [[-1.0]], accumulate=True)
        comb([Lvv.diagonal()], [e_v], [[-1.0]], accumulate=True)

        main.wait_stream(side)  # the compressed tensors from here on
        if "O^4V^2" in comp:  # sparse_cc_Woooo (:309-322)
            Wo = new(o, o, o, o)                                                  # [i,j,k,l]
            comb([Wo.permute(2, 3, 0, 1)], [ein2("lcki,jc->klij", E.ovoo, t1), ein2("kclj,ic->klij", E.ovoo, t1)])
            self._spmm(Tw, 0, 1, 2, 3, 1.0, E.ovov_cdkl, o * o, Wo, st, const="ovov_cdkl")  # 1323
            Woooo = Wo.permute(2, 3, 0, 1)                                        # (k,l,i,j)
            comb([Woooo], [ein2("kild,jd->klij", ein2("kcld,ic->kild", E.ovov, t1), t1)], accumulate=True)
            comb([Woooo], [E.oooo.permute(0, 2, 1, 3)], accumulate=True)
        else:
            Woooo = D.cc_Woooo(t1, t2, E)

        if "O^3V^3" in comp:  # sparse_cc_Wvoov / sparse_cc_Wvovo (:334-376)
            R = new(o * v * v, o)                          # R[(k,c,a), i] = sum_d (kc|ad) t_id
            mm(E.ovvv.view(o * v * v, v), t1.T, R, 1.0, 0.0, const="ovvv")
            Wp = new(v, o, o, v)                                                  # [a,i,k,c]
            Wvoov = Wp.permute(0, 2, 1, 3)                                        # (a,k,i,c)
            comb([Wvoov], [R.view(o, v, v, o).permute(2, 0, 3, 1), ein2("kcli,la->akic", E.ovoo, t1),
                           E.ovvo.permute(2, 0, 3, 1)], [[1.0, -1.0, 1.0]])
            self._spmm(Tw, 3, 0, 1, 2, -0.5, E.ovov, ov, Wp, st, const="ovov")                     # 0112
            self._spmm(Tw, 2, 0, 1, 3, 1.0, E.ovov_0313_0113, ov, Wp, st, const="ovov_0313_0113")  # 0313+0113
            comb([Wvoov], [ein2("lkci,la->akic", ein2("ldkc,id->lkci", E.ovov, t1), t1)], [[-1.0]],
                 accumulate=True)
            mm(E.ovvv_kacd.view(o * v * v, v), t1.T, R, 1.0, 0.0, const="ovvv_kacd")   # R[(k,a,c), i] = sum_d (kd|ac) t_id
            Wq = new(v, o, o, v)                                                  # [a,i,k,c]
            Wvovo = Wq.permute(0, 2, 3, 1)                                        # (a,k,c,i)
            comb([Wvovo], [R.view(o, v, v, o).permute(1, 0, 2, 3), ein2("lcki,la->akci", E.ovoo, t1),
                           E.oovv.permute(2, 0, 3, 1)], [[1.0, -1.0, 1.0]])
            self._spmm(Tw, 3, 0, 1, 2, -0.5, E.ovov_0312, ov, Wq, st, const="ovov_0312")          # 0312
            comb([Wvovo], [ein2("lkci,la->akci", ein2("lckd,id->lkci", E.ovov, t1), t1)], [[-1.0]],
                 accumulate=True)
            del R
        else:
            Wvoov = D.cc_Wvoov(t1, t2, E)
            Wvovo = D.cc_Wvovo(t1, t2, E)

        if "O^4V^2" in comp:
            comb([t2new], [ein2("lija,lb->ijab", ein2("klij,ka->lija", Woooo, t1), t1)], accumulate=True)
            Tp = new(v, v, o, o)                                                  # [a,b,i,j]
            comb([Tp], [t2new.permute(2, 3, 0, 1)])
            Wk = new(o, o, o, o)
            comb([Wk], [Woooo])
            self._spmm(T, 2, 3, 0, 1, 1.0, Wk, o * o, Tp, st)                     # 0101
            comb([t2new], [Tp.permute(2, 3, 0, 1)])
            del Tp, Wk
        else:
            tau = t2 + ein("ia,jb->ijab", t1, t1)
            t2new += ein("klij,klab->ijab", Woooo, tau)

        # Wvvvv terms (:207, :222-234)
        if self.wvvvv_t1t1 == "reference":
            # fricc/friccsd.py:222: einsum("abcd,ia,jb->ijab") sums c,d inside Wvvvv
            S = new(v, v)                                  # sum_cd Wvvvv[a,b,c,d]
            comb([S], [E.S0])
            mmf(E.U.T, t1, S, -1.0, 1.0)
            mmf(t1.T, E.U, S, -1.0, 1.0)
            comb([t2new], [], [[1.0]], prod=[S[None, None, :, :], t1[:, None, :, None], t1[None, :, None, :]],
                 accumulate=True)
            if "O^2V^4" in comp:
                if self.precision == "split":
                    # (ac|bd) rebuilt from the split factor on the tensor cores, FP32
                    # (every iteration into this solver's own buffer, or once
                    # into the block the solvers of these integrals share)
                    R = E.vvvv_rebuild
                    from .cholesky import dense_spmm, dense_spmm_ok
                    if self.split_sparse == "dense" and dense_spmm_ok(self._dims, 0, 1, 2, 3, v * v):
                        if self.rebuild_vvvv:  # into this solver's own buffer, every iteration
                            self._vvvv_bt = R.rebuild_split_b(self._vvvv_bt)
                            Bt = self._vvvv_bt
                        else:                  # once, shared by the solvers of these integrals
                            Bt = R.shared_split_b()
                        dense_spmm(T, self._dims, 0, 1, 2, 3, 1.0, Bt, v * v, t2new, self._tc_status)
                        W = None
                    elif self.rebuild_vvvv:
                        if self._vvvv_buf is None:
                            self._vvvv_buf = torch.empty(v * v, R.ldw, dtype=torch.float32, device=t2.device)
                        W = R.rebuild(self._vvvv_buf)
                    else:
                        W = R.W if R.W is not None else R.rebuild()
                    if W is not None:
                        L.check(self._spmm32(T, 0, 1, 2, 3, 1.0, _ptr(W), v * v, R.ldw, _ptr(t2new), st))
                else:
                    self._spmm(T, 0, 1, 2, 3, 1.0, E.vvvvT, v * v, t2new, st, const="vvvvT")  # (ac|bd) of 2323
                XY = D.zero(new(o, o, 2, o, v))
                self._spmm(T, 0, 1, 2, 3, 1.0, E.ovvv_XY, 2 * ov, XY, st, const="ovvv_XY")  # t1 parts
                XYv = XY.view(o * o, 2, o, v)
                t2v = t2new.view(o * o, v, v)
                mm(XYv[:, 0].transpose(1, 2), t1.unsqueeze(0).expand(o * o, o, v), t2v, -1.0, 1.0)  # -X t1
                mm(t1.T.unsqueeze(0).expand(o * o, v, o), XYv[:, 1], t2v, -1.0, 1.0)               # -t1 Y
                del XY
            else:
                WT = D.wvvvv_T(t1, E)
                t2new += ein("abcd,ijcd->ijab", WT.permute(2, 3, 0, 1), t2)
        else:
            WT = D.wvvvv_T(t1, E)
            Wvvvv = WT.permute(2, 3, 0, 1)
            t2new += ein("abcd,ic,jd->ijab", Wvvvv, t1, t1)
            if "O^2V^4" in comp:
                self._contract("2323", Wvvvv, T, t2new, st)
            else:
                t2new += ein("abcd,ijcd->ijab", Wvvvv, t2)

        tmpL = new(o, o, v, v)
        mm(Lvv.unsqueeze(0).expand(o * o, v, v), t2.view(o * o, v, v), tmpL.view(o * o, v, v), 1.0, 0.0)
        D.sym_add(t2new, tmpL, 1.0)                         # Lvv t2, :238-239
        mm(Loo.T, t2.view(o, o * v * v), tmpL.view(o, o * v * v), 1.0, 0.0)
        D.sym_add(t2new, tmpL, -1.0)                        # Loo t2, :240-241
        del tmpL

        if "O^3V^3" in comp:
            WA, WB, W2 = new(o, v, o, v), new(o, v, o, v), new(o, v, o, v)   # [k,c,i,a]
            comb([WA, WB, W2], [Wvoov.permute(1, 3, 2, 0), Wvovo.permute(1, 2, 3, 0)],
                 [[1.0, 0.0], [0.0, 1.0], [2.0, -1.0]])   # Wvoov(a,k,i,c), Wvovo(a,k,c,i), 2 WA - WB
            tmp = D.zero(new(o, v, o, v))                                     # [j,b,i,a]
            self._spmm(T, 1, 3, 0, 2, 1.0, W2, ov, tmp, st)                   # 1302 + 1202
            D.sym_add(t2new, tmp.permute(2, 0, 3, 1), 1.0)
            D.zero(tmp)
            self._spmm(T, 1, 2, 0, 3, 1.0, WA, ov, tmp, st)                   # 1303, [j,b,i,a]
            D.sym_add(t2new, tmp.permute(2, 0, 3, 1), -1.0)
            D.zero(tmp)
            self._spmm(T, 1, 2, 0, 3, 1.0, WB, ov, tmp, st)                   # 1203, [j,a,i,b]
            D.sym_add(t2new, tmp.permute(2, 0, 1, 3), -1.0)
            del WA, WB, W2, tmp
        else:
            tmp = 2 * ein("akic,kjcb->ijab", Wvoov, t2) - ein("akci,kjcb->ijab", Wvovo, t2)
            t2new += _sym(tmp)
            t2new -= _sym(ein("akic,kjbc->ijab", Wvoov, t2))
            t2new -= _sym(ein("bkci,kjac->ijab", Wvovo, t2))

        # denominators + energy + step norm (:281-284, :418-427)
        t1o = t1 if t1_old is None else t1_old
        t2o = t2 if t2_old is None else t2_old
        L.check(self.lib.fricc_energy_update(_ptr(t1new), _ptr(t2new), _ptr(C["eia"]), _ptr(fov),
                                             _ptr(E.ovov), _ptr(t1o.contiguous()), _ptr(t2o.contiguous()), o, v,
                                             _ptr(t1new), _ptr(t2new), _ptr(self._res), st))
        return t1new, t2new

    def _timed(self, verbose, compress):
        """Run one compression; with ``verbose``, print the reference's phase
        table for it (src/fri_utils.cpp:509-519) from CUDA events at its
        phase boundaries."""
        if not verbose:
            return compress()
        from .py_rccsd import print_phase_table
        L.check(self.lib.fricc_phase_timing_set(1))
        sec = (ctypes.c_double * 5)()
        try:
            h = compress()
            L.check(self.lib.fricc_phase_timing_read(sec))
        finally:
            self.lib.fricc_phase_timing_set(0)
        print_phase_table(list(sec))
        return h

    def _constants(self, o, v):
        """Per-solver constants of the iteration, built once: contiguous
        Fock blocks, the shifted orbital energies and the denominator
        matrix eia = e_i - e_a (fricc/friccsd.py:83, :281-284)."""
        key = (o, v)
        if getattr(self, "_const_key", None) != key:
            E = self.eris
            e_o = E.mo_energy[:o].contiguous()
            e_v = (E.mo_energy[o:] + self.level_shift).contiguous()
            self._const = {"foo": E.fock[:o, :o].contiguous(), "fvv": E.fock[o:, o:].contiguous(),
                           "fov": E.fock[:o, o:].contiguous(), "e_o": e_o, "e_v": e_v,
                           "eia": (e_o[:, None] - e_v[None, :]).contiguous()}
            self._const_key = key
        return self._const

    def _w_source(self, t2):
        """T2, or after burn-in in the unbiased mode its running average
        Y = X/it + (it-1)/it Y (it = iterations past burn-in; it = 0 and 1 both
        restart from X), evaluated in the reference's operation order."""
        s = self.settings
        if not s.get("unbiased", False) or self._iter < s["burn_in"]:
            return t2
        it = self._iter - s["burn_in"]
        if it == 0 or self._t2_avg is None:
            self._t2_avg = t2.clone()
        else:
            # a tensor divisor: division by a host scalar may be done as a
            # multiply by its reciprocal, which rounds differently from X/it
            div = torch.full((1,), float(it), dtype=t2.dtype, device=t2.device)
            self._t2_avg = t2 / div + ((it - 1) / it) * self._t2_avg
        return self._t2_avg

    def reset_average(self):
        """Restart the iteration count (and so the burn-in) of the unbiased mode."""
        self._iter = 0
        self._t2_avg = None

    def _handles_in_use(self):
        return [h for h in (self._sp, self._sp_w) if h.h.value]

    def read_energy(self):
        """E_corr and the step norm of the last update (waits for it); raises
        if one of its compressions failed (a probability above 1)."""
        r = self._res[:2].cpu()
        for h in self._handles_in_use():
            L.check(self.lib.fricc_sp_status(h.h))
        if self.precision == "split":
            self.eris.vvvv_rebuild.check()
            if int(self._tc_status.item()):
                raise L.FriccError(5, "split-precision GEMM: a bounded tensor-core pipeline wait gave up")
        self.last_energy, self.last_normt = float(r[0]), float(r[1])
        return self.last_energy, self.last_normt

    def energy(self, t1, t2):
        return D.ccsd_energy(t1, t2, self.eris)

    def update_amps_host(self, t1_host: np.ndarray, t2_host: np.ndarray, rn=None, out=None):
        """End-to-end step: numpy amplitudes in (copied to HBM), numpy out.

        The results are copied into ``out`` (a pair of float64 arrays) when
        given; otherwise into one of two solver-owned page-locked buffer pairs
        used in turn, so a result stays valid until the call after next (feed
        it back as the next input, as the iteration loop does)."""
        t1 = torch.from_numpy(t1_host).to(self.eris.device, non_blocking=True)
        t2 = torch.from_numpy(t2_host).to(self.eris.device, non_blocking=True)
        t1n, t2n = self.update_amps(t1, t2, rn=rn)
        if out is None:
            bufs = getattr(self, "_host_out", None)
            if bufs is None or bufs[0][1].shape != t2n.shape:
                bufs = [(torch.empty(t1n.shape, dtype=t1n.dtype, pin_memory=True),
                         torch.empty(t2n.shape, dtype=t2n.dtype, pin_memory=True)) for _ in range(2)]
                self._host_out, self._host_turn = bufs, 0
            h1, h2 = bufs[self._host_turn]
            self._host_turn ^= 1
        else:
            h1, h2 = torch.from_numpy(out[0]), torch.from_numpy(out[1])
        h1.copy_(t1n, non_blocking=True)
        h2.copy_(t2n, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        return h1.numpy(), h2.numpy()

    def kernel(self, t1=None, t2=None, max_cycle=50, tol=1e-8, tolnormt=1e-6, callback=None):
        """The iteration loop of fricc/friccsd.py:379-456 (no DIIS).
        Returns (converged, e_corr, t1, t2, energies)."""
        if t1 is None or t2 is None:
            raise ValueError("pass initial amplitudes (e.g. MP2) as device tensors")
        eold, ecc = 0.0, self.energy(t1, t2)
        energies = []
        conv = False
        for it in range(max_cycle):
            t1, t2 = self.update_amps(t1, t2)
            eold = ecc
            ecc, normt = self.read_energy()
            energies.append(ecc)
            if callback is not None:
                callback(it, t1, t2, ecc)
            if abs(ecc - eold) < tol and normt < tolnormt:
                conv = True
                break
            if np.isnan(ecc - eold) or abs(ecc - eold) > 1e5:
                conv = False
                break
        return conv, ecc, t1, t2, energies
