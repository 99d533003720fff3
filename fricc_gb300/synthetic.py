"""Seeded synthetic closed-shell systems for FRI-CCSD.

A system is defined by (nocc, nvir, naux, sigma, seed):

* orbital energies: occupied uniform in [-1.5, -0.3] Eh, virtual uniform in
  [0.2, 3.0] Eh, each sorted ascending; the Fock matrix is diagonal, so the
  occupied-virtual block f_ov is zero;
* two-electron integrals in chemists' notation
  (pq|rs) = sum_P L[P,p,q] L[P,r,s], with L symmetric in (p,q) and its
  independent entries drawn N(0, sigma^2 / naux): a normalised factor, so
  the diagonal integrals (pq|pq) are ~sigma^2 whatever naux is.  With entries
  N(0, sigma^2) as such, the named workloads are far outside the regime in
  which undamped CCSD iterates converge (o10v40: E_MP2 = -105 Eh,
  max |t2| = 0.44, and CCSD without any compression diverges within three
  iterations; a 1/naux^(1/4) scale still leaves o20v100 oscillating between
  -2.7 and -4.5 Eh).  With the normalised factor every workload converges
  (o10v40: E_corr -0.0025875 Eh, o20v100: -0.0079092 Eh, FRI fluctuations
  ~1e-7 Eh) with the same sizes and the same work per iteration;
* amplitudes start at T1 = 0 and T2 = MP2, t_ijab = (ia|jb) / (e_i+e_j-e_a-e_b).

These are the stand-in inputs for the reference's molecular runs (PySCF
SCF on real molecules is not available); the named workloads below carry the
sizes used by the tests and the benchmark.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

# Named workloads: nocc, nvir, naux, sigma, m (kept nonzeros), iterations.
WORKLOADS = {
    "o10v40": dict(nocc=10, nvir=40, naux=200, sigma=0.05, m=20000, iters=20),
    "o30v150": dict(nocc=30, nvir=150, naux=900, sigma=0.03, m=2_000_000, iters=30),
    "o20v100x64": dict(nocc=20, nvir=100, naux=600, sigma=0.04, m=200_000, iters=30, replicas=64),
    "o40v200": dict(nocc=40, nvir=200, naux=1200, sigma=0.025, m=3_200_000, iters=40),
}


@dataclass
class SyntheticSystem:
    nocc: int
    nvir: int
    naux: int
    sigma: float
    seed: int = 0
    mo_energy: np.ndarray = field(init=False)
    L: np.ndarray = field(init=False)  # (naux, nmo, nmo), symmetric in the last two

    def __post_init__(self):
        rng = np.random.default_rng(self.seed)
        eo = np.sort(rng.uniform(-1.5, -0.3, self.nocc))
        ev = np.sort(rng.uniform(0.2, 3.0, self.nvir))
        self.mo_energy = np.concatenate([eo, ev])
        nmo = self.nmo
        A = rng.standard_normal((self.naux, nmo, nmo)) * (self.sigma / self.naux ** 0.5)
        up = np.triu(A)
        self.L = up + np.transpose(np.triu(A, 1), (0, 2, 1))

    @property
    def nmo(self) -> int:
        return self.nocc + self.nvir

    @property
    def fock(self) -> np.ndarray:
        return np.diag(self.mo_energy)

    def _sl(self, c):
        return slice(0, self.nocc) if c == "o" else slice(self.nocc, self.nmo)

    def eri(self, block: str) -> np.ndarray:
        """Chemists'-notation block, e.g. eri('ovov')[i,a,j,b] = (ia|jb), FP64 numpy."""
        p, q, r, s = (self._sl(c) for c in block)
        Lpq = self.L[:, p, q]
        Lrs = self.L[:, r, s]
        n1, n2 = Lpq.shape[1:]
        n3, n4 = Lrs.shape[1:]
        g = Lpq.reshape(self.naux, -1).T @ Lrs.reshape(self.naux, -1)
        return g.reshape(n1, n2, n3, n4)

    def mp2_amplitudes(self):
        o = self.nocc
        eo, ev = self.mo_energy[:o], self.mo_energy[o:]
        eia = eo[:, None] - ev[None, :]
        eijab = eia[:, None, :, None] + eia[None, :, None, :]
        t2 = self.eri("ovov").transpose(0, 2, 1, 3) / eijab
        t1 = np.zeros((o, self.nvir))
        return t1, np.ascontiguousarray(t2)


class DeviceSystem:
    """The same recipe drawn on the GPU (torch's Philox generator seeded with
    ``seed``): the same distributions and sizes as ``SyntheticSystem``, but
    not the same numbers.  A request server uses it for every arm it
    compares, so that drawing a few hundred million normals on the host does
    not stand in front of every solve."""

    def __init__(self, nocc, nvir, naux, sigma, seed=0, device="cuda"):
        import torch
        self.nocc, self.nvir, self.naux, self.sigma, self.seed = int(nocc), int(nvir), int(naux), sigma, seed
        dev = torch.device(device)
        g = torch.Generator(device=dev)
        g.manual_seed(int(seed))
        f64 = torch.float64
        eo = torch.sort(torch.rand(self.nocc, generator=g, device=dev, dtype=f64) * 1.2 - 1.5).values
        ev = torch.sort(torch.rand(self.nvir, generator=g, device=dev, dtype=f64) * 2.8 + 0.2).values
        self.mo_energy = torch.cat([eo, ev])
        nmo = self.nmo
        A = torch.randn(self.naux, nmo, nmo, generator=g, device=dev, dtype=f64) * (sigma / self.naux ** 0.5)
        self.L = torch.triu(A) + torch.triu(A, 1).transpose(1, 2)

    @property
    def nmo(self) -> int:
        return self.nocc + self.nvir

    @property
    def fock(self):
        import torch
        return torch.diag(self.mo_energy)


def make_system(name: str, seed: int = 0) -> SyntheticSystem:
    w = WORKLOADS[name]
    return SyntheticSystem(w["nocc"], w["nvir"], w["naux"], w["sigma"], seed)
