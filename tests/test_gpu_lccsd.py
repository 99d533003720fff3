"""The FRI-LCCSD iteration on the GPU (fricc_gb300/frilccsd.py) against the
reference's own fricc/frilccsd.py trajectories (tests/golden/lccsd.npz) and
the oracle (oracle/lccsd_oracle.py), step by step with the same amplitudes
and draws: both compress identically (bit for bit), so only rounding in the
algebra differs.  Bound: |dE_corr| <= 1e-10 Eh per step; amplitudes to
1e-12 relative (FP64) or 1e-10 relative (FP32-pair "df64")."""
import numpy as np
import pytest
import torch

from conftest import golden

pytestmark = pytest.mark.gpu

BASE = {"compression": "fri", "sampling_method": "systematic", "verbose": False,
        "compressed_contractions": ["O^2V^4", "O^3V^3", "O^4V^2"]}
VARIANTS = (("shared", False, False), ("independent", True, False), ("lccd", False, True))


def _golden_system():
    from fricc_gb300.synthetic import SyntheticSystem
    g = golden("lccsd.npz")
    s = SyntheticSystem.__new__(SyntheticSystem)
    s.nocc, s.L, s.mo_energy = int(g["nocc"]), g["L"], g["mo_energy"]
    s.naux, s.nvir = s.L.shape[0], s.mo_energy.size - int(g["nocc"])
    s.sigma, s.seed = 0.0, 0
    return g, s


def _settings(m, indep, lccd, comp=None):
    d = dict(BASE, m_keep=m, **{"Independent Compressions": indep, "LCCD": lccd})
    if comp is not None:
        d["compressed_contractions"] = comp
    return d


@pytest.mark.parametrize("precision", ["fp64", "df64"])
@pytest.mark.parametrize("name,indep,lccd", VARIANTS)
def test_lccsd_golden_teacher_forced(gpulib, name, indep, lccd, precision):
    from fricc_gb300.frilccsd import FRILCCSDGPU
    from fricc_gb300.rccsd_dense import DeviceERIs
    g, s = _golden_system()
    m = int(g["m"])
    gs = FRILCCSDGPU(DeviceERIs.from_system(s), _settings(m, indep, lccd), precision=precision)
    per = gs.n_draws
    assert per == (6 if indep else 1)
    rn = list(g[f"{name}_rn"])
    rtol = 1e-12 if precision == "fp64" else 1e-10
    for it in range(len(g[f"{name}_energies"])):
        t1 = torch.from_numpy(g[f"{name}_t1"][it]).cuda()
        t2 = torch.from_numpy(g[f"{name}_t2"][it]).cuda()
        t1n, t2n = gs.update_amps(t1, t2, rn=rn[per * it: per * it + per])
        e, _ = gs.read_energy()
        assert abs(e - g[f"{name}_energies"][it]) < 1e-10, (it, e)
        ref2 = g[f"{name}_t2"][it + 1]
        assert np.abs(t2n.cpu().numpy() - ref2).max() < rtol * np.abs(ref2).max()
        ref1 = g[f"{name}_t1"][it + 1]
        assert np.abs(t1n.cpu().numpy() - ref1).max() <= rtol * max(np.abs(ref1).max(), 1e-300)
        if lccd:
            assert not torch.any(t1n)


@pytest.mark.parametrize("comp", [[], ["O^2V^4"], ["O^3V^3"], ["O^4V^2"]])
def test_lccsd_partial_compression_vs_oracle(gpulib, oracle, comp):
    """Terms left dense take the einsum branches of fricc/frilccsd.py."""
    from oracle import lccsd_oracle as LO
    from oracle import pyscf_standin as P
    from fricc_gb300.frilccsd import FRILCCSDGPU
    from fricc_gb300.rccsd_dense import DeviceERIs
    from fricc_gb300.synthetic import SyntheticSystem
    s = SyntheticSystem(6, 24, 120, 0.05, 3)
    m = 5000
    eris = P.make_eris(s)
    for precision in ("fp64", "df64"):
        gs = FRILCCSDGPU(DeviceERIs.from_system(s), _settings(m, False, False, comp), precision=precision)
        t1h, t2h = s.mp2_amplitudes()
        t1h = t1h + 1e-3 * np.random.default_rng(1).standard_normal(t1h.shape)  # exercise the t1 terms
        t1n, t2n = gs.update_amps(torch.from_numpy(t1h).cuda(), torch.from_numpy(t2h).cuda(), rn=[0.37])
        draws = iter([0.37])
        o1, o2 = LO.update_amps(_settings(m, False, False, comp), t1h, t2h, eris, rn_draw=lambda: next(draws))
        e, _ = gs.read_energy()
        assert abs(e - LO.lin_cc_energy(o1, o2, eris)) < 1e-10
        assert np.abs(t2n.cpu().numpy() - o2).max() < 1e-10 * np.abs(o2).max()
        assert np.abs(t1n.cpu().numpy() - o1).max() < 1e-10 * np.abs(o1).max()


def test_lccsd_kernel_converges(gpulib):
    """The loop with the linearised energy converges on o10v40 (largest-m
    compression keeps it deterministic) to the oracle's energy."""
    from oracle import lccsd_oracle as LO
    from oracle import pyscf_standin as P
    from fricc_gb300.frilccsd import FRILCCSDGPU
    from fricc_gb300.rccsd_dense import DeviceERIs
    from fricc_gb300.synthetic import SyntheticSystem
    s = SyntheticSystem(10, 40, 200, 0.05, 0)
    settings = dict(_settings(160000, False, False), compression="largest")
    gs = FRILCCSDGPU(DeviceERIs.from_system(s), settings)
    t1h, t2h = s.mp2_amplitudes()
    conv, e, t1, t2, energies = gs.kernel(torch.from_numpy(t1h).cuda(), torch.from_numpy(t2h).cuda(),
                                          max_cycle=40, tol=1e-10, tolnormt=1e-7)
    assert conv
    c2, e2, _, _, _ = LO.kernel(settings, P.make_eris(s), t1h, t2h, max_cycle=40, tol=1e-10, tolnormt=1e-7)
    assert c2 and abs(e - e2) < 1e-10
