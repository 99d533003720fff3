"""Independent spin-orbital CCSD update (test helper).

Written from the spin-orbital CCSD equations with the intermediates of
Stanton & Gauss, J. Chem. Phys. 94, 4334 (1991) (also Crawford & Schaefer,
Rev. Comp. Chem. 14, 33 (2000)), for a diagonal Fock matrix.  Spin orbitals
are ordered (p alpha, p beta) for each spatial p, occupied first.  It shares
no code with the closed-shell equations it checks.
"""
import numpy as np


def spin_integrals(system):
    o, n = system.nocc, system.nmo
    full = np.einsum("Ppq,Prs->pqrs", system.L, system.L)  # (pq|rs)
    sp = np.repeat(np.arange(n), 2)
    sg = np.tile([0, 1], n)
    g = full[np.ix_(sp, sp, sp, sp)].transpose(0, 2, 1, 3)  # <pq|rs> = (pr|qs)
    mask = (sg[:, None, None, None] == sg[None, None, :, None]) & (sg[None, :, None, None] == sg[None, None, None, :])
    g = g * mask
    A = g - g.transpose(0, 1, 3, 2)  # <pq||rs>
    e = system.mo_energy[sp]
    return A, e, 2 * o


def spin_update(system, t1, t2):
    """One Jacobi update (t1, t2) -> (t1', t2') of spin-orbital CCSD."""
    A, e, no = spin_integrals(system)
    O, V = slice(0, no), slice(no, A.shape[0])
    fov = np.zeros((no, A.shape[0] - no))
    Dia = e[O][:, None] - e[V][None, :]
    Dijab = Dia[:, None, :, None] + Dia[None, :, None, :]
    oovv = A[O, O, V, V]
    tt = t2 + 0.5 * (np.einsum("ia,jb->ijab", t1, t1) - np.einsum("ib,ja->ijab", t1, t1))
    tau = t2 + np.einsum("ia,jb->ijab", t1, t1) - np.einsum("ib,ja->ijab", t1, t1)
    Fae = (-0.5 * np.einsum("me,ma->ae", fov, t1) + np.einsum("mf,mafe->ae", t1, A[O, V, V, V])
           - 0.5 * np.einsum("mnaf,mnef->ae", tt, oovv))
    Fmi = (0.5 * np.einsum("ie,me->mi", t1, fov) + np.einsum("ne,mnie->mi", t1, A[O, O, O, V])
           + 0.5 * np.einsum("inef,mnef->mi", tt, oovv))
    Fme = fov + np.einsum("nf,mnef->me", t1, oovv)
    Wmnij = (A[O, O, O, O] + np.einsum("je,mnie->mnij", t1, A[O, O, O, V])
             - np.einsum("ie,mnje->mnij", t1, A[O, O, O, V]) + 0.25 * np.einsum("ijef,mnef->mnij", tau, oovv))
    Wabef = (A[V, V, V, V] - np.einsum("mb,amef->abef", t1, A[V, O, V, V])
             + np.einsum("ma,bmef->abef", t1, A[V, O, V, V]) + 0.25 * np.einsum("mnab,mnef->abef", tau, oovv))
    Wmbej = (A[O, V, V, O] + np.einsum("jf,mbef->mbej", t1, A[O, V, V, V])
             - np.einsum("nb,mnej->mbej", t1, A[O, O, V, O])
             - np.einsum("jnfb,mnef->mbej", 0.5 * t2 + np.einsum("jf,nb->jnfb", t1, t1), oovv))
    r1 = (fov + np.einsum("ie,ae->ia", t1, Fae) - np.einsum("ma,mi->ia", t1, Fmi)
          + np.einsum("imae,me->ia", t2, Fme) - np.einsum("nf,naif->ia", t1, A[O, V, O, V])
          - 0.5 * np.einsum("imef,maef->ia", t2, A[O, V, V, V]) - 0.5 * np.einsum("mnae,nmei->ia", t2, A[O, O, V, O]))
    x = np.einsum("ijae,be->ijab", t2, Fae - 0.5 * np.einsum("mb,me->be", t1, Fme))
    r2 = oovv + x - x.transpose(0, 1, 3, 2)
    x = np.einsum("imab,mj->ijab", t2, Fmi + 0.5 * np.einsum("je,me->mj", t1, Fme))
    r2 -= x - x.transpose(1, 0, 2, 3)
    r2 += 0.5 * np.einsum("mnab,mnij->ijab", tau, Wmnij) + 0.5 * np.einsum("ijef,abef->ijab", tau, Wabef)
    x = np.einsum("imae,mbej->ijab", t2, Wmbej) - np.einsum("ie,ma,mbej->ijab", t1, t1, A[O, V, V, O])
    r2 += x - x.transpose(1, 0, 2, 3) - x.transpose(0, 1, 3, 2) + x.transpose(1, 0, 3, 2)
    x = np.einsum("ie,abej->ijab", t1, A[V, V, V, O])
    r2 += x - x.transpose(1, 0, 2, 3)
    x = np.einsum("ma,mbij->ijab", t1, A[O, V, O, O])
    r2 -= x - x.transpose(0, 1, 3, 2)
    return r1 / Dia, r2 / Dijab
