"""Oracle FRI-CCSD iteration: a CPU restatement of fricc/friccsd.py.

TEST INFRASTRUCTURE ONLY: used by the tests, the smoke check and the
CPU-baseline leg of bench.py to check or time the GPU iteration.  The product
never imports it.

``update_amps`` restates fricc/friccsd.py:29-301 (two FRI compressions, the
sparse W intermediates :309-376, the eleven compressed terms, the dense rest
and the denominators) on numpy, with the compressions and contractions taken
from the C oracle (oracle/fri_oracle.c) and the dense CCSD algebra from
oracle/pyscf_standin.py.  ``kernel`` restates the iteration loop :379-456.

With ``settings["unbiased"]`` the W-intermediate compression takes, once
``burn_in`` iterations have run, the running average of the T2 inputs
instead of T2 (fricc/friccsd.py:108-136).  The reference reads an iteration
counter ``cc._iter`` that nothing defines; here it is ``state["iter"]``, the
number of updates run before this one, kept with the average in ``state``.

The reference's T2 update adds ``einsum("abcd,ia,jb->ijab", Wvvvv, t1, t1)``
(fricc/friccsd.py:222), which sums c and d inside Wvvvv instead of
contracting them with t1 (CCSD has ``ic,jd``).  Parity means reproducing
that term; ``wvvvv_t1t1="ccsd"`` selects the textbook term instead.
"""
from __future__ import annotations

import time

import numpy as np

from . import fri_oracle as FO
from . import pyscf_standin as PS

ALLOWED_CONTRACTIONS = ("O^2V^4", "O^3V^3", "O^4V^2")
DEFAULT_SETTINGS = {
    "m_keep": 1000,
    "compression": "fri",
    "sampling_method": "systematic",
    "verbose": False,
    "compressed_contractions": ["O^2V^4", "O^3V^3", "O^4V^2"],
    "burn_in": 100,
    "unbias": False,
}


def pivotal_tensor(sparse, x, m, rn_draw):
    """A pivotal compression drawing from rn_draw: a GlibcRand-like stream
    (history()/set_history()) is copied, the copy supplies up to one draw per
    element, and the stream is then advanced by the draws consumed; anything
    else means libc's own rand(), as the reference draws."""
    if hasattr(rn_draw, "history"):
        from fricc_gb300.rng import GlibcRand
        probe = GlibcRand(1)
        probe.set_history(rn_draw.history())
        draws = np.array([probe.uniform() for _ in range(x.size)])
        T = sparse.SparseTensor4d(x, x.shape, m, "fri", "pivotal", draws=draws)
        for _ in range(T.draws_used):
            rn_draw.rand()
        return T
    return sparse.SparseTensor4d(x, x.shape, m, "fri", "pivotal")


def _sym(x):
    """x_ijab + x_jiba"""
    return x + x.transpose(1, 0, 3, 2)


def update_amps(settings, t1, t2, eris, rn_draw=FO.libc_rand_uniform, sparse=FO,
                level_shift=0.0, timings=None, wvvvv_t1t1="reference", state=None):
    """One FRI-CCSD amplitude update; returns (t1new, t2new).

    rn_draw() supplies the uniform draw of each systematic compression, in
    call order (compression #1 for the T2 terms, #2 for the W intermediates).
    """
    m = int(settings["m_keep"])
    if m > t2.size or m == 0:
        raise ValueError("Bad m_keep value! The following condition wasn't met 0 < m_keep <= t2.size")
    comp = settings["compressed_contractions"]
    tim = {} if timings is None else timings
    nocc, nvir = t1.shape
    fock = eris.fock
    e_o = eris.mo_energy[:nocc]
    e_v = eris.mo_energy[nocc:] + level_shift
    fov = fock[:nocc, nocc:].copy()
    t2 = np.ascontiguousarray(t2)

    def compress(x=t2):
        kind = settings["compression"]
        if kind == "fri" and settings["sampling_method"] == "pivotal":
            return pivotal_tensor(sparse, x, m, rn_draw)
        rn = rn_draw() if kind == "fri" else None
        return sparse.SparseTensor4d(x, x.shape, m, kind, settings["sampling_method"],
                                     settings["verbose"], rn=rn)

    state = {} if state is None else state
    n_done = state.get("iter", 0)

    tc = time.perf_counter()
    t2_sp = compress()
    t2_sp_w = None
    if "O^3V^3" in comp or "O^4V^2" in comp:
        if not settings.get("unbiased", False) or n_done < settings.get("burn_in", 100):
            t2_sp_w = compress()
        else:  # running average Y(t+1) = (1 - 1/t) Y(t) + X(t)/t, as written at :121-127
            it = n_done - settings.get("burn_in", 100)
            if it == 0:
                state["t2_avg"] = t2
            else:
                state["t2_avg"] = t2 / it + (it - 1) / it * state["t2_avg"]
            t2_sp_w = compress(state["t2_avg"])
    state["iter"] = n_done + 1
    tim["compress"] = time.perf_counter() - tc

    Foo = PS.cc_Foo(t1, t2, eris)
    Fvv = PS.cc_Fvv(t1, t2, eris)
    Fov = PS.cc_Fov(t1, t2, eris)
    Foo[np.diag_indices(nocc)] -= e_o
    Fvv[np.diag_indices(nvir)] -= e_v

    # T1 equation (fricc/friccsd.py:153-176)
    t1new = -2 * np.einsum("kc,ka,ic->ia", fov, t1, t1)
    t1new += np.einsum("ac,ic->ia", Fvv, t1)
    t1new += -np.einsum("ki,ka->ia", Foo, t1)
    t1new += 2 * np.einsum("kc,kica->ia", Fov, t2)
    t1new += -np.einsum("kc,ikca->ia", Fov, t2)
    t1new += np.einsum("kc,ic,ka->ia", Fov, t1, t1)
    t1new += fov.conj()
    t1new += 2 * np.einsum("kcai,kc->ia", eris.ovvo, t1)
    t1new += -np.einsum("kiac,kc->ia", eris.oovv, t1)
    ovvv = eris.get_ovvv()
    ein = PS.einsum
    t1new += 2 * ein("kdac,ikcd->ia", ovvv, t2)
    t1new += -ein("kcad,ikcd->ia", ovvv, t2)
    t1new += 2 * ein("kdac,kd,ic->ia", ovvv, t1, t1)
    t1new += -ein("kcad,kd,ic->ia", ovvv, t1, t1)
    ovoo = eris.ovoo
    t1new += -2 * ein("lcki,klac->ia", ovoo, t2)
    t1new += ein("kcli,klac->ia", ovoo, t2)
    t1new += -2 * ein("lcki,lc,ka->ia", ovoo, t1, t1)
    t1new += ein("kcli,lc,ka->ia", ovoo, t1, t1)

    # T2 driver terms (:179-187)
    tmp2 = ein("kibc,ka->abic", eris.oovv, -t1)
    tmp2 += ovvv.conj().transpose(1, 3, 0, 2)
    t2new = _sym(ein("abic,jc->ijab", tmp2, t1))
    tmp2 = ein("kcai,jc->akij", eris.ovvo, t1)
    tmp2 += ovoo.transpose(1, 3, 0, 2).conj()
    t2new -= _sym(ein("akij,kb->ijab", tmp2, t1))
    t2new += eris.ovov.conj().transpose(0, 2, 1, 3)

    Loo = PS.Loo(t1, t2, eris)
    Lvv = PS.Lvv(t1, t2, eris)
    Loo[np.diag_indices(nocc)] -= e_o
    Lvv[np.diag_indices(nvir)] -= e_v

    def timed(term, W, T, out):
        t = time.perf_counter()
        sparse.contract_DTSpT(W, T, out, term)
        tim[term] = time.perf_counter() - t

    ovov = eris.ovov
    if "O^4V^2" in comp:  # sparse_cc_Woooo (:309-322)
        Woooo = ein("lcki,jc->klij", ovoo, t1)
        Woooo += ein("kclj,ic->klij", ovoo, t1)
        timed("1323", ovov, t2_sp_w, Woooo)
        Woooo += ein("kcld,ic,jd->klij", ovov, t1, t1)
        Woooo += eris.oooo.transpose(0, 2, 1, 3)
    else:
        Woooo = PS.cc_Woooo(t1, t2, eris)

    if "O^3V^3" in comp:  # sparse_cc_Wvoov (:334-360), sparse_cc_Wvovo (:363-376)
        Wvoov = ein("kcad,id->akic", ovvv, t1)
        Wvoov -= ein("kcli,la->akic", ovoo, t1)
        Wvoov += eris.ovvo.transpose(2, 0, 3, 1)
        timed("0112", ovov, t2_sp_w, Wvoov)
        timed("0313", ovov, t2_sp_w, Wvoov)
        timed("0113", ovov, t2_sp_w, Wvoov)
        Wvoov -= ein("ldkc,id,la->akic", ovov, t1, t1)
        Wvovo = ein("kdac,id->akci", ovvv, t1)
        Wvovo -= ein("lcki,la->akci", ovoo, t1)
        Wvovo += eris.oovv.transpose(2, 0, 3, 1)
        timed("0312", ovov, t2_sp_w, Wvovo)
        Wvovo -= ein("lckd,id,la->akci", ovov, t1, t1)
    else:
        Wvoov = PS.cc_Wvoov(t1, t2, eris)
        Wvovo = PS.cc_Wvovo(t1, t2, eris)

    # cc_Wvvvv (:325-331)
    Wvvvv = ein("kdac,kb->abcd", ovvv, -t1)
    Wvvvv -= ein("kcbd,ka->abcd", ovvv, t1)
    Wvvvv += PS._get_vvvv(eris).transpose(0, 2, 1, 3)

    if "O^4V^2" in comp:
        t2new += ein("klij,ka,lb->ijab", Woooo, t1, t1)
        timed("0101", Woooo, t2_sp, t2new)
    else:
        tau = t2 + np.einsum("ia,jb->ijab", t1, t1)
        t2new += ein("klij,klab->ijab", Woooo, tau)

    if wvvvv_t1t1 == "reference":
        t2new += ein("abcd,ia,jb->ijab", Wvvvv, t1, t1)
    else:
        t2new += ein("abcd,ic,jd->ijab", Wvvvv, t1, t1)
    if "O^2V^4" in comp:
        timed("2323", Wvvvv, t2_sp, t2new)
    else:
        t2new += ein("abcd,ijcd->ijab", Wvvvv, t2)

    t2new += _sym(ein("ac,ijcb->ijab", Lvv, t2))
    t2new -= _sym(ein("ki,kjab->ijab", Loo, t2))

    if "O^3V^3" in comp:
        tmp = np.zeros_like(t2new)
        timed("1302", Wvoov, t2_sp, tmp)
        timed("1202", Wvovo, t2_sp, tmp)
        t2new += _sym(tmp)
        tmp = np.zeros_like(t2new)
        timed("1303", Wvoov, t2_sp, tmp)
        t2new -= _sym(tmp)
        tmp = np.zeros_like(t2new)
        timed("1203", Wvovo, t2_sp, tmp)
        t2new -= _sym(tmp)
    else:
        tmp = 2 * ein("akic,kjcb->ijab", Wvoov, t2)
        tmp -= ein("akci,kjcb->ijab", Wvovo, t2)
        t2new += _sym(tmp)
        t2new -= _sym(ein("akic,kjbc->ijab", Wvoov, t2))
        t2new -= _sym(ein("bkci,kjac->ijab", Wvovo, t2))

    eia = e_o[:, None] - e_v
    eijab = PS.direct_sum("ia,jb->ijab", eia, eia)
    t1new /= eia
    t2new /= eijab
    return t1new, t2new


def kernel(settings, eris, t1=None, t2=None, max_cycle=50, tol=1e-8, tolnormt=1e-6,
           rn_draw=FO.libc_rand_uniform, sparse=FO, callback=None, wvvvv_t1t1="reference"):
    """The FRI-CCSD loop of fricc/friccsd.py:379-456 (no DIIS); returns
    (converged, e_corr, t1, t2, energies)."""
    if t1 is None or t2 is None:
        t1, t2 = PS.mp2_guess(eris)
    eold = 0.0
    state = {}
    ecc = PS.ccsd_energy(t1, t2, eris)
    energies = []
    conv = False
    for it in range(max_cycle):
        t1n, t2n = update_amps(settings, t1, t2, eris, rn_draw=rn_draw, sparse=sparse,
                               wvvvv_t1t1=wvvvv_t1t1, state=state)
        normt = np.linalg.norm(PS.amplitudes_to_vector(t1n, t2n) - PS.amplitudes_to_vector(t1, t2))
        t1, t2 = t1n, t2n
        eold, ecc = ecc, PS.ccsd_energy(t1, t2, eris)
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
