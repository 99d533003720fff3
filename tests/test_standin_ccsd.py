"""Pins the dense CCSD algebra that stands in for PySCF (oracle/pyscf_standin.py
and fricc_gb300/rccsd_dense.py share its equations) against an independent
spin-orbital CCSD written from the Stanton-Gauss equations (tests/spin_ccsd.py).

The reference's T2 update (fricc/friccsd.py:222) adds
einsum("abcd,ia,jb->ijab", Wvvvv, t1, t1), which is not the CCSD term
einsum("abcd,ic,jd->ijab", ...): with the CCSD term the closed-shell update
equals the spin-orbital one to rounding; with the reference's term it
differs at second order in t1.  Both facts are checked."""
import numpy as np

from spin_ccsd import spin_update


def _setup(o=2, v=4, seed=3):
    from oracle import pyscf_standin as P
    from fricc_gb300.synthetic import SyntheticSystem
    s = SyntheticSystem(o, v, 40, 0.08, seed)
    return s, P.make_eris(s)


def _to_spin(t1, t2):
    o, v = t1.shape
    T1 = np.zeros((2 * o, 2 * v))
    T1[0::2, 0::2] = t1
    T1[1::2, 1::2] = t1
    T2 = np.zeros((2 * o, 2 * o, 2 * v, 2 * v))
    T2[0::2, 1::2, 0::2, 1::2] = t2
    T2[1::2, 0::2, 1::2, 0::2] = t2
    T2[0::2, 1::2, 1::2, 0::2] = -t2.transpose(0, 1, 3, 2)
    T2[1::2, 0::2, 0::2, 1::2] = -t2.transpose(0, 1, 3, 2)
    aa = t2 - t2.transpose(0, 1, 3, 2)
    T2[0::2, 0::2, 0::2, 0::2] = aa
    T2[1::2, 1::2, 1::2, 1::2] = aa
    return T1, T2


def test_closed_shell_update_matches_spin_orbital(oracle):
    from oracle import ccsd_oracle as CO
    s, eris = _setup()
    rng = np.random.default_rng(5)
    o, v = s.nocc, s.nvir
    t2 = rng.standard_normal((o, o, v, v)) * 0.05
    t2 = 0.5 * (t2 + t2.transpose(1, 0, 3, 2))
    t1 = rng.standard_normal((o, v)) * 0.01
    settings = {"m_keep": 10, "compression": "largest", "sampling_method": "systematic",
                "compressed_contractions": [], "verbose": False}
    S1, S2 = spin_update(s, *_to_spin(t1, t2))
    n1, n2 = CO.update_amps(settings, t1, t2, eris, wvvvv_t1t1="ccsd")
    assert np.abs(S1[0::2, 0::2] - n1).max() < 1e-15
    assert np.abs(S2[0::2, 1::2, 0::2, 1::2] - n2).max() < 1e-15
    r1, r2 = CO.update_amps(settings, t1, t2, eris)  # the reference's term
    assert np.abs(r1 - n1).max() < 1e-15
    assert np.abs(S2[0::2, 1::2, 0::2, 1::2] - r2).max() > 1e-8


def test_ccsd_energy_and_mp2(oracle):
    from oracle import pyscf_standin as P
    s, eris = _setup()
    t1, t2 = P.mp2_guess(eris)
    o = s.nocc
    ovov = eris.ovov
    e = s.mo_energy
    emp2 = 0.0
    for i in range(o):
        for j in range(o):
            for a in range(s.nvir):
                for b in range(s.nvir):
                    d = e[i] + e[j] - e[o + a] - e[o + b]
                    emp2 += ovov[i, a, j, b] * (2 * ovov[i, a, j, b] - ovov[i, b, j, a]) / d
    assert abs(P.ccsd_energy(t1, t2, eris) - emp2) < 1e-14
