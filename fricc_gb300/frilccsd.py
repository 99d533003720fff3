"""GPU FRI-LCCSD: the linearised-CCSD iteration of fri-cc's fricc/frilccsd.py.

``FRILCCSDGPU`` runs ``update_amps`` (fricc/frilccsd.py:27-261) or, with the
setting ``"Independent Compressions"``, ``update_amps_independent_compressions``
(:264-501) on the device, and the loop of fricc/friccsd.py:379-456 with the
linearised energy ``lin_cc_energy`` (:504-522):

* one FRI compression of T2 per iteration shared by the six sparse terms, or
  six independent compressions (one draw each, in the order 2323, 0101,
  1302, 1202, 1303, 1203), bit for bit the reference's;
* the sparse terms contract the compressed T2 with bare integral blocks
  ((ac|bd), (ki|lj), (kc|ai), (ki|ac)), which are constants of the solve:
  their layouts (and, for precision "df64", their float-pair forms) are
  built once on the DeviceERIs;
* 1302 and 1202 share one pass over a combined W' when they share a
  compression;
* the dense terms (Fock terms, the O^2V^3 T1 term, the t1 driver terms) as
  GEMMs; ``"LCCD": True`` zeroes t1 on entry and keeps t1new at zero
  (:124-127);
* the denominators, the linearised energy and the step norm fused in
  ``fricc_energy_update_lin``.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib as L
from . import rccsd_dense as D
from .friccsd import ALLOWED_CONTRACTIONS, FRICCSDGPU, _check_sampling, _compress, _Handle, _ptr, _sym
from .py_rccsd import libc_uniform

DEFAULT_SETTINGS = {
    "m_keep": 1000,
    "compression": "fri",
    "sampling_method": "systematic",
    "verbose": False,
    "compressed_contractions": ["O^2V^4", "O^3V^3", "O^4V^2"],
    "LCCD": False,
    "Independent Compressions": False,
}
SPARSE_ORDER = ("2323", "0101", "1302", "1202", "1303", "1203")


class FRILCCSDGPU(FRICCSDGPU):
    def __init__(self, eris: D.DeviceERIs, fri_settings=None, level_shift=0.0, rn_draw=libc_uniform,
                 precision="fp64"):
        s = dict(DEFAULT_SETTINGS)
        s.update(fri_settings or {})
        for c in s["compressed_contractions"]:
            if c not in ALLOWED_CONTRACTIONS:
                raise ValueError(f"Contraction ({c}) is not supported!")
        if s["compression"] not in L.COMPRESSION:
            raise ValueError(f"The compression method you chose ({s['compression']}) isn't supported")
        _check_sampling(s, rn_draw)
        if precision not in ("fp64", "df64"):
            raise ValueError("precision must be 'fp64' or 'df64'")
        self.settings = s
        self.eris = eris
        self.level_shift = float(level_shift)
        self.rn_draw = rn_draw
        self.precision = precision
        self._df = precision == "df64"
        self._tuner = None  # the shared sparse-term dispatcher's autotuner (not used here)
        self.lib = L.load()
        eris.prepare_linear()
        if precision == "df64":
            eris.prepare_splits(("vvvvT",) + D.DeviceERIs.LIN_BLOCKS)
        self.independent = bool(s["Independent Compressions"])
        self._handles = [_Handle() for _ in range(len(SPARSE_ORDER) if self.independent else 1)]
        self._res = torch.zeros(4, dtype=torch.float64, device=eris.device)
        self.timings = {}
        self.last_energy = None
        self.last_normt = None

    @property
    def n_draws(self):
        """Uniform draws one iteration takes as rn (one per systematic FRI
        compression; pivotal sampling draws its own)."""
        s = self.settings
        return len(self._handles) if s["compression"] == "fri" and s["sampling_method"] == "systematic" else 0

    def update_amps(self, t1, t2, rn=None, t1_old=None, t2_old=None):
        """One FRI-LCCSD iteration on device tensors; returns (t1new, t2new).

        rn: the uniform draw of each compression (1, or 6 with independent
        compressions); default rn_draw().  read_energy() then gives the
        linearised E_corr of (t1new, t2new) and the step norm against
        (t1_old, t2_old) (default: the inputs)."""
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
        e_o = E.mo_energy[:o]
        e_v = E.mo_energy[o:] + self.level_shift
        fov = E.fock[:o, o:]
        ein = torch.einsum
        mm = D.gemm_df if self.precision == "df64" else D.gemm_f64

        def ein2(spec, A_, B_):
            return D.einsum_df(spec, A_, B_, gemm=mm)
        f64, dev = t2.dtype, t2.device
        if rn is None:
            rn = [self.rn_draw() for _ in range(self.n_draws)]
        if self.n_draws and len(rn) != len(self._handles):
            raise ValueError(f"update_amps: {len(self._handles)} draws expected, got {len(rn)}")
        rn = list(rn) if self.n_draws else [0.0] * len(self._handles)
        Ts = [_compress(h, t2, m, s, r, self.rn_draw, st) for h, r in zip(self._handles, rn)]
        T = dict(zip(SPARSE_ORDER, Ts if self.independent else Ts * len(SPARSE_ORDER)))

        Foo = E.fock[:o, :o].clone()
        Fvv = E.fock[o:, o:].clone()
        Foo.diagonal().sub_(e_o)
        Fvv.diagonal().sub_(e_v)
        lccd = bool(s["LCCD"])
        t1_in = t1
        # T1 (fricc/frilccsd.py:124-156)
        if lccd:
            t1 = torch.zeros_like(t1)
            t1new = torch.zeros_like(t1)
        else:
            t1new = fov + t1 @ Fvv.T - Foo.T @ t1
            t1new += 2 * ein("kcai,kc->ia", E.ovvo, t1) - ein("kiac,kc->ia", E.oovv, t1)
            t1new = t1new.contiguous()
            mm(t2.view(o, o * v * v), E.G_t1.view(o * v * v, v), t1new, 1.0, 1.0)  # terms 5: O^2V^3
            t1new -= ein2("lcki,klac->ia", E.g_ovoo, t2)                              # term 6
            t1new += 2 * ein("kc,kica->ia", fov, t2) - ein("kc,ikca->ia", fov, t2)    # term 7

        # T2 (:158-239)
        t2new = E.ovov.permute(0, 2, 1, 3).contiguous()
        tmp = torch.empty_like(t2)
        mm(Foo.T, t2.view(o, o * v * v), tmp.view(o, o * v * v), 1.0, 0.0)           # Foo t2
        t2new -= _sym(tmp)
        mm(Fvv.unsqueeze(0).expand(o * o, v, v), t2.view(o * o, v, v), tmp.view(o * o, v, v), 1.0, 0.0)
        t2new += _sym(tmp)                                                           # Fvv t2
        del tmp
        if "O^2V^4" in comp:
            self._spmm(T["2323"], 0, 1, 2, 3, 1.0, E.vvvvT, v * v, t2new, st, const="vvvvT")
        else:
            t2new += ein2("cdab,ijcd->ijab", E.vvvvT, t2)
        if "O^4V^2" in comp:
            Tp = t2new.permute(2, 3, 0, 1).contiguous()                                  # [a,b,i,j]
            self._spmm(T["0101"], 2, 3, 0, 1, 1.0, E.oooo_klij, o * o, Tp, st, const="oooo_klij")
            t2new.copy_(Tp.permute(2, 3, 0, 1))
            del Tp
        else:
            t2new += ein2("klij,klab->ijab", E.oooo_klij, t2)
        if "O^3V^3" in comp:
            tmp = torch.zeros(o, v, o, v, dtype=f64, device=dev)                        # [j,b,i,a]
            if T["1302"] is T["1202"]:
                self._spmm(T["1302"], 1, 3, 0, 2, 1.0, E.lin_W2AB, ov, tmp, st, const="lin_W2AB")
            else:
                self._spmm(T["1302"], 1, 3, 0, 2, 2.0, E.lin_WA, ov, tmp, st, const="lin_WA")
                self._spmm(T["1202"], 1, 3, 0, 2, -1.0, E.lin_WB, ov, tmp, st, const="lin_WB")
            t2new += _sym(tmp.permute(2, 0, 3, 1))
            tmp.zero_()
            self._spmm(T["1303"], 1, 2, 0, 3, 1.0, E.lin_WA, ov, tmp, st, const="lin_WA")     # [j,b,i,a]
            t2new -= _sym(tmp.permute(2, 0, 3, 1))
            tmp.zero_()
            self._spmm(T["1203"], 1, 2, 0, 3, 1.0, E.lin_WB, ov, tmp, st, const="lin_WB")     # [j,a,i,b]
            t2new -= _sym(tmp.permute(2, 0, 1, 3))
            del tmp
        else:
            WA = E.lin_WA.permute(3, 0, 2, 1)          # Wvoov[a,k,i,c]
            WB = E.lin_WB.permute(3, 0, 1, 2)          # Wvovo[a,k,c,i]
            t2new += _sym(2 * ein2("akic,kjcb->ijab", WA, t2) - ein2("akci,kjcb->ijab", WB, t2))
            t2new -= _sym(ein2("akic,kjbc->ijab", WA, t2))
            t2new -= _sym(ein2("bkci,kjac->ijab", WB, t2))
        if not lccd:
            R = torch.empty(o * v * o, v, dtype=f64, device=dev)
            mm(E.ovoo.view(o * v * o, o), t1, R, 1.0, 0.0)                              # R[(i,a,j),b] = sum_k (ia|jk) t_kb
            t2new -= _sym(R.view(o, v, o, v).permute(0, 2, 1, 3))                       # term 7
            R = torch.empty(o * v * v, o, dtype=f64, device=dev)
            mm(E.ovvv_iabc.view(o * v * v, v), t1.T, R, 1.0, 0.0)                       # R[(i,a,b),j] = sum_c (ia|bc) t_jc
            t2new += _sym(R.view(o, v, v, o).permute(0, 3, 1, 2))                       # term 8
            del R

        eia = (e_o[:, None] - e_v[None, :]).contiguous()
        t1new = t1new.contiguous()
        t2new = t2new.contiguous()
        t1o = t1_in if t1_old is None else t1_old
        t2o = t2 if t2_old is None else t2_old
        L.check(self.lib.fricc_energy_update_lin(_ptr(t1new), _ptr(t2new), _ptr(eia), _ptr(fov.contiguous()),
                                                 _ptr(E.ovov), _ptr(t1o.contiguous()), _ptr(t2o.contiguous()), o, v,
                                                 _ptr(t1new), _ptr(t2new), _ptr(self._res), st))
        return t1new, t2new

    def _handles_in_use(self):
        return [h for h in self._handles if h.h.value]

    def energy(self, t1, t2):
        return D.lin_cc_energy(t1, t2, self.eris)
