"""Dense closed-shell CCSD pieces of one FRI-CCSD iteration, on the GPU (FP64).

These are the parts of fricc/friccsd.py:update_amps that the reference
delegates to PySCF (``rintermediates`` cc_Foo, cc_Fvv, cc_Fov, Loo, Lvv and
the dense W intermediates, the CCSD energy) written from the closed-shell
CCSD equations (Hirata et al., J. Chem. Phys. 120, 2581 (2004)), with torch
tensors on the device.  torch is the plumbing here: the contractions below
are cuBLAS GEMMs; the hot path (compression, sparse terms, denominators) is
the CUDA library.

Integral blocks, chemists' notation: ovov[i,a,j,b] = (ia|jb),
oovv[i,j,a,b] = (ij|ab), ovvo[i,a,b,j] = (ia|bj), ovoo[i,a,j,k] = (ia|jk),
ovvv[i,a,b,c] = (ia|bc), oooo[i,j,k,l] = (ij|kl); the vvvv block is kept
only as vvvvT[c,d,a,b] = (ac|bd), the layout the O^2V^4 term streams.
"""
from __future__ import annotations

import numpy as np
import torch

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
        else:
            self.vvvvT = vvvv.permute(1, 3, 0, 2).contiguous()  # [c,d,a,b] = (ac|bd)
        del vvvv
        self._derive()

    def _derive(self):
        # layouts reused every iteration
        self.g_ovov = 2.0 * self.ovov - self.ovov.permute(0, 3, 2, 1)    # 2(kc|ld) - (kd|lc)
        self.ovvv_kcda = self.ovvv.permute(0, 3, 1, 2).contiguous()       # [k,c,d,a] = (kd|ac)
        self.ovvv_cdkb = self.ovvv.permute(1, 3, 0, 2).contiguous()       # [c,d,k,b] = (kc|bd)

    @classmethod
    def from_system(cls, system, device="cuda"):
        """Build every block on the device from the Cholesky factor of a SyntheticSystem."""
        dev = torch.device(device)
        L = torch.from_numpy(system.L).to(dev, torch.float64)
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

        blocks = {k: blk(k) for k in ("oooo", "ovoo", "ovov", "oovv", "ovvo", "ovvv")}
        Lvv = L[:, sl["v"], sl["v"]]
        v = system.nvir
        # vvvvT[c,d,a,b] = (ac|bd) = sum_P L[P,a,c] L[P,b,d]
        Lca = Lvv.permute(0, 2, 1).reshape(naux, v * v)  # [P, (c,a)]
        Ldb = Lvv.permute(0, 2, 1).reshape(naux, v * v)  # [P, (d,b)]
        X = (Lca.T @ Ldb).reshape(v, v, v, v)            # [c,a,d,b]
        blocks["vvvvT"] = X.permute(0, 2, 1, 3).contiguous()
        del X
        return cls(torch.from_numpy(system.fock), torch.from_numpy(system.mo_energy), o, blocks, device)

    def to_numpy_blocks(self):
        """Host copies in the stand-in layout (for checking against the oracle)."""
        out = {k: getattr(self, k).cpu().numpy() for k in ("oooo", "ovoo", "ovov", "oovv", "ovvo", "ovvv")}
        out["vvvv"] = self.vvvvT.permute(2, 0, 3, 1).contiguous().cpu().numpy()  # (ab|cd)
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


def Loo(t1, t2, E):
    o = t1.shape[0]
    fov = E.fock[:o, o:]
    g = 2.0 * E.ovoo - E.ovoo.permute(2, 1, 0, 3)  # [l,c,k,i]: 2(lc|ki) - (kc|li)
    return cc_Foo(t1, t2, E) + fov @ t1.T + ein("lcki,lc->ki", g, t1)


def Lvv(t1, t2, E):
    o = t1.shape[0]
    fov = E.fock[:o, o:]
    g = 2.0 * E.ovvv - E.ovvv.permute(0, 3, 2, 1)  # [k,d,a,c]: 2(kd|ac) - (kc|ad)
    return cc_Fvv(t1, t2, E) - t1.T @ fov + ein("kdac,kd->ac", g, t1)


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


def ccsd_energy(t1, t2, E):
    o = t1.shape[0]
    fov = E.fock[:o, o:]
    tau = t2 + ein("ia,jb->ijab", t1, t1)
    return float(2.0 * (fov * t1).sum() + ein("ijab,iajb->", tau, E.g_ovov))
