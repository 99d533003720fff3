"""Oracle FRI-LCCSD iteration: a CPU restatement of fricc/frilccsd.py.

TEST INFRASTRUCTURE ONLY: used by the tests to check the GPU FRI-LCCSD
iteration.  The product never imports it.

Linearised CCSD (Taube and Bartlett, J. Chem. Phys. 130, 144112 (2009),
eqs. 13 and 15, the reference's citation) keeps only the terms of the CCSD
residual that are linear in the amplitudes, so every W the compressed T2 is
contracted with is a bare integral block:
  2323  W = (ac|bd)         0101  W = (ki|lj)
  1302  W = (kc|ai)         1202  W = (ki|ac)   (also 1303 / 1203)
``update_amps`` restates fricc/frilccsd.py:27-261 (one compression shared by
all sparse terms) and, with ``independent=True``, :264-501 (six
compressions, one per sparse term, in the order 2323, 0101, 1302, 1202,
1303, 1203, each drawing one uniform).  ``lccd=True`` is the reference's
"LCCD" setting (:124-127): t1 is zeroed on entry and t1new stays zero.
``lin_cc_energy`` restates :504-522 and ``kernel`` the loop of
fricc/friccsd.py:379-456 with that energy.
"""
from __future__ import annotations

import numpy as np

from . import fri_oracle as FO
from . import pyscf_standin as PS

SPARSE_ORDER = ("2323", "0101", "1302", "1202", "1303", "1203")


def _sym(x):
    """x_ijab + x_jiba"""
    return x + x.transpose(1, 0, 3, 2)


def lin_cc_energy(t1, t2, eris):
    """2 sum f_ia t1_ia + sum t2_ijab (2 (ia|jb) - (ib|ja)) (fricc/frilccsd.py:504-522)."""
    nocc = t1.shape[0]
    e = 2.0 * np.einsum("ia,ia", eris.fock[:nocc, nocc:], t1)
    e += 2.0 * np.einsum("ijab,iajb", t2, eris.ovov)
    e += -np.einsum("ijab,ibja", t2, eris.ovov)
    return float(e)


def update_amps(settings, t1, t2, eris, rn_draw=FO.libc_rand_uniform, sparse=FO, level_shift=0.0,
                independent=False, lccd=False):
    """One FRI-LCCSD amplitude update; returns (t1new, t2new)."""
    m = int(settings["m_keep"])
    if m > t2.size or m == 0:
        raise ValueError("Bad m_keep value! The following condition wasn't met 0 < m_keep <= t2.size")
    comp = settings["compressed_contractions"]
    nocc, nvir = t1.shape
    fock = eris.fock
    e_o = eris.mo_energy[:nocc]
    e_v = eris.mo_energy[nocc:] + level_shift
    t2 = np.ascontiguousarray(t2)

    def compress():
        kind = settings["compression"]
        if kind == "fri" and settings["sampling_method"] == "pivotal":
            from .ccsd_oracle import pivotal_tensor
            return pivotal_tensor(sparse, t2, m, rn_draw)
        rn = rn_draw() if kind == "fri" else None
        return sparse.SparseTensor4d(t2, t2.shape, m, kind, settings["sampling_method"],
                                     settings["verbose"], rn=rn)

    if independent:
        sp = dict(zip(SPARSE_ORDER, [compress() for _ in SPARSE_ORDER]))
    else:
        one = compress()
        sp = {k: one for k in SPARSE_ORDER}

    Foo = fock[:nocc, :nocc].copy()
    Fvv = fock[nocc:, nocc:].copy()
    Fov = fock[:nocc, nocc:].copy()
    Foo[np.diag_indices(nocc)] -= e_o
    Fvv[np.diag_indices(nvir)] -= e_v
    ovoo = eris.ovoo
    ovvv = eris.get_ovvv()
    ein = PS.einsum

    # T1 (:124-156)
    t1new = np.zeros_like(t1)
    if lccd:
        t1 = np.zeros_like(t1)
    else:
        t1new += Fov.conj()
        t1new += np.einsum("ac,ic->ia", Fvv, t1)
        t1new += -np.einsum("ki,ka->ia", Foo, t1)
        t1new += 2 * np.einsum("kcai,kc->ia", eris.ovvo, t1)
        t1new += -np.einsum("kiac,kc->ia", eris.oovv, t1)
        t1new += 2 * ein("kdac,ikcd->ia", ovvv, t2)
        t1new += -ein("kcad,ikcd->ia", ovvv, t2)
        t1new += -2 * ein("lcki,klac->ia", ovoo, t2)
        t1new += ein("kcli,klac->ia", ovoo, t2)
        t1new += 2 * np.einsum("kc,kica->ia", Fov, t2)
        t1new += -np.einsum("kc,ikca->ia", Fov, t2)

    # T2 (:158-247)
    t2new = eris.ovov.conj().transpose(0, 2, 1, 3).copy()
    t2new -= _sym(ein("ki,kjab->ijab", Foo, t2))
    t2new += _sym(ein("ac,ijcb->ijab", Fvv, t2))
    Woooo = eris.oooo.transpose(0, 2, 1, 3)
    Wvoov = eris.ovvo.transpose(2, 0, 3, 1)
    Wvovo = eris.oovv.transpose(2, 0, 3, 1)
    Wvvvv = PS._get_vvvv(eris).transpose(0, 2, 1, 3)
    if "O^2V^4" in comp:
        sparse.contract_DTSpT(Wvvvv, sp["2323"], t2new, "2323")
    else:
        t2new += ein("abcd,ijcd->ijab", Wvvvv, t2)
    if "O^4V^2" in comp:
        sparse.contract_DTSpT(Woooo, sp["0101"], t2new, "0101")
    else:
        t2new += ein("klij,klab->ijab", Woooo, t2)
    if "O^3V^3" in comp:
        tmp = np.zeros_like(t2new)
        sparse.contract_DTSpT(Wvoov, sp["1302"], tmp, "1302")
        sparse.contract_DTSpT(Wvovo, sp["1202"], tmp, "1202")
        t2new += _sym(tmp)
        tmp = np.zeros_like(t2new)
        sparse.contract_DTSpT(Wvoov, sp["1303"], tmp, "1303")
        t2new -= _sym(tmp)
        tmp = np.zeros_like(t2new)
        sparse.contract_DTSpT(Wvovo, sp["1203"], tmp, "1203")
        t2new -= _sym(tmp)
    else:
        tmp = 2 * ein("akic,kjcb->ijab", Wvoov, t2) - ein("akci,kjcb->ijab", Wvovo, t2)
        t2new += _sym(tmp)
        t2new -= _sym(ein("akic,kjbc->ijab", Wvoov, t2))
        t2new -= _sym(ein("bkci,kjac->ijab", Wvovo, t2))
    t2new -= _sym(ein("akij,kb->ijab", ovoo.transpose(1, 3, 0, 2).conj(), t1))
    t2new += _sym(ein("iabc,jc->ijab", ovvv.conj(), t1))

    eia = e_o[:, None] - e_v
    t1new /= eia
    t2new /= eia[:, None, :, None] + eia[None, :, None, :]
    return t1new, t2new


def kernel(settings, eris, t1=None, t2=None, max_cycle=50, tol=1e-8, tolnormt=1e-6,
           rn_draw=FO.libc_rand_uniform, sparse=FO, independent=False, lccd=False, callback=None):
    """The FRI-LCCSD loop (fricc/friccsd.py:379-456 with lin_cc_energy, no
    DIIS); returns (converged, e_corr, t1, t2, energies)."""
    if t1 is None or t2 is None:
        t1, t2 = PS.mp2_guess(eris)
    ecc = lin_cc_energy(t1, t2, eris)
    energies = []
    conv = False
    for it in range(max_cycle):
        t1n, t2n = update_amps(settings, t1, t2, eris, rn_draw=rn_draw, sparse=sparse,
                               independent=independent, lccd=lccd)
        normt = np.linalg.norm(PS.amplitudes_to_vector(t1n, t2n) - PS.amplitudes_to_vector(t1, t2))
        t1, t2 = t1n, t2n
        eold, ecc = ecc, lin_cc_energy(t1, t2, eris)
        energies.append(ecc)
        if callback is not None:
            callback(it, t1, t2, ecc)
        if abs(ecc - eold) < tol and normt < tolnormt:
            conv = True
            break
        if np.isnan(ecc - eold) or abs(ecc - eold) > 1e5:
            break
    return conv, ecc, t1, t2, energies
