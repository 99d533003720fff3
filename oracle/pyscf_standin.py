"""A minimal stand-in for the parts of PySCF that fri-cc's FRI-CCSD driver calls.

TEST INFRASTRUCTURE ONLY.  PySCF (a third-party, unpinned dependency of the
reference: its CI installs the latest release) is not available here.  This
module restates, from the closed-shell CCSD equations (Hirata et al.,
J. Chem. Phys. 120, 2581 (2004), the reference cited at fricc/friccsd.py:56),
exactly the PySCF entry points that fricc/friccsd.py uses, so that

* the reference's own ``fricc/friccsd.py`` can run unmodified in this
  container (``install()`` registers fake ``pyscf`` modules), which is how the
  golden iteration vectors in tests/golden/ are produced, and
* the oracle driver (oracle/ccsd_oracle.py) shares the same dense algebra.

Call sites covered (fricc/friccsd.py): ``ccsd.CCSD`` / ``ccsd._ChemistsERIs``
(:5,29-34,62,462), ``lib.einsum`` / ``lib.direct_sum`` / ``lib.logger``
(:6-7,64,282), ``rintermediates`` cc_Foo, cc_Fvv, cc_Fov, Loo, Lvv, cc_Woooo,
cc_Wvoov, cc_Wvovo, _get_vvvv (:144-146,189-190,197,204-205,330), and the
CCSD energy, MP2 initial guess and amplitude packing used by ``kernel``
(:396,402,418-427).

Integral blocks are chemists' notation: ovov[i,a,j,b] = (ia|jb),
oovv[i,j,a,b] = (ij|ab), ovvo[i,a,b,j] = (ia|bj), ovoo[i,a,j,k] = (ia|jk),
ovvv[i,a,b,c] = (ia|bc), oooo[i,j,k,l] = (ij|kl), vvvv[a,b,c,d] = (ab|cd).
"""
from __future__ import annotations

import sys
import time
import types

import numpy as np


# --------------------------------------------------------------------------
# lib
# --------------------------------------------------------------------------
def einsum(subscripts, *operands, **kw):
    kw.pop("order", None)
    return np.einsum(subscripts, *operands, optimize=True)


def direct_sum(subscripts, a, b):
    """Outer sum of two operands with disjoint indices, e.g. 'ia,jb->ijab'."""
    ins, out = subscripts.replace(" ", "").split("->")
    sa, sb = ins.split(",")
    full = sa + sb
    A = a.reshape(a.shape + (1,) * len(sb))
    B = b.reshape((1,) * len(sa) + b.shape)
    s = A + B
    return np.ascontiguousarray(np.transpose(s, [full.index(c) for c in out]))


class _Logger:
    def __init__(self, verbose=0):
        self.verbose = verbose
        self.records = []

    def _rec(self, kind, msg, *args):
        text = msg % args if args else msg
        self.records.append((kind, text))
        if self.verbose >= 4 and kind in ("info", "warn"):
            print(text)

    def debug(self, msg, *args):
        self._rec("debug", msg, *args)

    def info(self, msg, *args):
        self._rec("info", msg, *args)

    def warn(self, msg, *args):
        self._rec("warn", msg, *args)

    note = info

    def timer(self, msg, *cput):
        return (time.process_time(), time.perf_counter())


def new_logger(obj=None, verbose=None):
    return _Logger(getattr(obj, "verbose", 0) if verbose is None else verbose)


class DIIS:  # kernel() only tests isinstance against it; DIIS is skipped (:425-426)
    pass


# --------------------------------------------------------------------------
# ccsd
# --------------------------------------------------------------------------
class _ChemistsERIs:
    def __init__(self, fock, mo_energy, nocc, blocks):
        self.fock = fock
        self.mo_energy = mo_energy
        self.nocc = nocc
        for k, v in blocks.items():
            setattr(self, k, v)

    def get_ovvv(self):
        return self.ovvv


def make_eris(system) -> _ChemistsERIs:
    """Integral blocks of a fricc_gb300.synthetic.SyntheticSystem as numpy arrays."""
    blocks = {b: system.eri(b) for b in ("oooo", "ovoo", "ovov", "oovv", "ovvo", "ovvv", "vvvv")}
    return _ChemistsERIs(system.fock, system.mo_energy, system.nocc, blocks)


def ccsd_energy(t1, t2, eris):
    """E_corr = 2 sum f_ia t_ia + sum tau_ijab [2 (ia|jb) - (ib|ja)], tau = t2 + t1 t1."""
    nocc = t1.shape[0]
    fov = eris.fock[:nocc, nocc:]
    tau = t2 + np.einsum("ia,jb->ijab", t1, t1)
    g = 2.0 * eris.ovov - eris.ovov.transpose(0, 3, 2, 1)  # [i,a,j,b]
    return 2.0 * np.einsum("ia,ia", fov, t1) + np.einsum("ijab,iajb", tau, g)


def mp2_guess(eris):
    nocc = eris.nocc
    e = eris.mo_energy
    eia = e[:nocc, None] - e[None, nocc:]
    t1 = eris.fock[:nocc, nocc:] / eia
    t2 = eris.ovov.transpose(0, 2, 1, 3) / direct_sum("ia,jb->ijab", eia, eia)
    return t1, np.ascontiguousarray(t2)


def amplitudes_to_vector(t1, t2):
    """t1 followed by the lower triangle (with diagonal) of t2 viewed as an (ia, jb) matrix."""
    nocc, nvir = t1.shape
    nov = nocc * nvir
    M = t2.transpose(0, 2, 1, 3).reshape(nov, nov)
    return np.concatenate([t1.ravel(), M[np.tril_indices(nov)]])


class CCSD:
    """Just the attributes and methods fricc/friccsd.py's kernel/update_amps read."""

    def __init__(self, eris=None, fri_settings=None, verbose=0):
        self.max_cycle = 50
        self.conv_tol = 1e-7
        self.conv_tol_normt = 1e-5
        self.level_shift = 0.0
        self.diis = False
        self.diis_file = None
        self.diis_space = 6
        self.incore_complete = True
        self.verbose = verbose
        self.eris = eris
        self._fri_settings = dict(fri_settings or {})

    @property
    def fri_settings(self):
        return self._fri_settings

    def ao2mo(self, mo_coeff=None):
        return self.eris

    def get_init_guess(self, eris=None):
        return mp2_guess(eris or self.eris)

    def energy(self, t1, t2, eris):
        return ccsd_energy(t1, t2, eris)

    def amplitudes_to_vector(self, t1, t2):
        return amplitudes_to_vector(t1, t2)


# --------------------------------------------------------------------------
# rintermediates (closed-shell CCSD intermediates)
# --------------------------------------------------------------------------
def _g_ovov(eris):
    """2 (kc|ld) - (kd|lc), indexed [k,c,l,d]."""
    return 2.0 * eris.ovov - eris.ovov.transpose(0, 3, 2, 1)


def cc_Foo(t1, t2, eris):
    nocc = t1.shape[0]
    tt = t2 + np.einsum("ic,ld->ilcd", t1, t1)
    return eris.fock[:nocc, :nocc] + einsum("kcld,ilcd->ki", _g_ovov(eris), tt)


def cc_Fvv(t1, t2, eris):
    nocc = t1.shape[0]
    tt = t2 + np.einsum("ka,ld->klad", t1, t1)
    return eris.fock[nocc:, nocc:] - einsum("kcld,klad->ac", _g_ovov(eris), tt)


def cc_Fov(t1, t2, eris):
    nocc = t1.shape[0]
    return eris.fock[:nocc, nocc:] + einsum("kcld,ld->kc", _g_ovov(eris), t1)


def Loo(t1, t2, eris):
    nocc = t1.shape[0]
    fov = eris.fock[:nocc, nocc:]
    ovoo = eris.ovoo
    g = 2.0 * ovoo - ovoo.transpose(2, 1, 0, 3)  # [l,c,k,i] -> 2(lc|ki) - (kc|li)
    return cc_Foo(t1, t2, eris) + fov @ t1.T + einsum("lcki,lc->ki", g, t1)


def Lvv(t1, t2, eris):
    nocc = t1.shape[0]
    fov = eris.fock[:nocc, nocc:]
    ovvv = eris.get_ovvv()
    g = 2.0 * ovvv - ovvv.transpose(0, 3, 2, 1)  # [k,d,a,c] -> 2(kd|ac) - (kc|ad)
    return cc_Fvv(t1, t2, eris) - t1.T @ fov + einsum("kdac,kd->ac", g, t1)


def cc_Woooo(t1, t2, eris):
    ovoo, ovov = eris.ovoo, eris.ovov
    W = einsum("lcki,jc->klij", ovoo, t1)
    W += einsum("kclj,ic->klij", ovoo, t1)
    W += einsum("kcld,ijcd->klij", ovov, t2 + np.einsum("ic,jd->ijcd", t1, t1))
    W += eris.oooo.transpose(0, 2, 1, 3)
    return W


def cc_Wvoov(t1, t2, eris):
    ovvv, ovoo, ovov = eris.get_ovvv(), eris.ovoo, eris.ovov
    W = einsum("kcad,id->akic", ovvv, t1)
    W -= einsum("kcli,la->akic", ovoo, t1)
    W += eris.ovvo.transpose(2, 0, 3, 1)
    W -= 0.5 * einsum("ldkc,ilda->akic", ovov, t2)
    W -= 0.5 * einsum("lckd,ilad->akic", ovov, t2)
    W += einsum("ldkc,ilad->akic", ovov, t2)
    W -= einsum("ldkc,id,la->akic", ovov, t1, t1)
    return W


def cc_Wvovo(t1, t2, eris):
    ovvv, ovoo, ovov = eris.get_ovvv(), eris.ovoo, eris.ovov
    W = einsum("kdac,id->akci", ovvv, t1)
    W -= einsum("lcki,la->akci", ovoo, t1)
    W += eris.oovv.transpose(2, 0, 3, 1)
    W -= 0.5 * einsum("lckd,ilda->akci", ovov, t2)
    W -= einsum("lckd,id,la->akci", ovov, t1, t1)
    return W


def _get_vvvv(eris):
    return eris.vvvv


# --------------------------------------------------------------------------
# fake module registration
# --------------------------------------------------------------------------
def install():
    """Register fake ``pyscf``, ``pyscf.lib``, ``pyscf.lib.logger``,
    ``pyscf.cc``, ``pyscf.cc.ccsd`` and ``pyscf.cc.rintermediates`` modules."""
    if "pyscf" in sys.modules and getattr(sys.modules["pyscf"], "_fricc_standin", False):
        return sys.modules["pyscf"]
    pyscf = types.ModuleType("pyscf")
    pyscf._fricc_standin = True
    lib = types.ModuleType("pyscf.lib")
    logger = types.ModuleType("pyscf.lib.logger")
    diis = types.ModuleType("pyscf.lib.diis")
    cc = types.ModuleType("pyscf.cc")
    ccsd = types.ModuleType("pyscf.cc.ccsd")
    imd = types.ModuleType("pyscf.cc.rintermediates")

    logger.new_logger = new_logger
    logger.process_clock = time.process_time
    logger.perf_counter = time.perf_counter
    logger.WARN = 2
    diis.DIIS = DIIS
    lib.einsum = einsum
    lib.direct_sum = direct_sum
    lib.logger = logger
    lib.diis = diis
    ccsd.CCSD = CCSD
    ccsd._ChemistsERIs = _ChemistsERIs
    for f in (cc_Foo, cc_Fvv, cc_Fov, Loo, Lvv, cc_Woooo, cc_Wvoov, cc_Wvovo, _get_vvvv):
        setattr(imd, f.__name__, f)
    cc.ccsd = ccsd
    cc.rintermediates = imd
    pyscf.lib = lib
    pyscf.cc = cc
    for name, mod in (("pyscf", pyscf), ("pyscf.lib", lib), ("pyscf.lib.logger", logger),
                      ("pyscf.lib.diis", diis), ("pyscf.cc", cc), ("pyscf.cc.ccsd", ccsd),
                      ("pyscf.cc.rintermediates", imd)):
        sys.modules[name] = mod
    return pyscf
