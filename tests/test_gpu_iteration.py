"""The whole FRI-CCSD iteration on the GPU against the oracle iteration
(oracle/ccsd_oracle.py, itself pinned to the reference's fricc/friccsd.py by
tests/golden/iteration.npz).

Parity is checked step by step ("teacher forced"): both sides get the same
amplitudes and the same two uniform draws, so both compress identically (bit
for bit) and the only differences are FP64 rounding in the dense and sparse
algebra.  Bound: |dE_corr| <= 1e-10 Eh per step; amplitudes to 1e-12
relative.  Free-running trajectories are compared too while they stay on the
same sample path."""
import numpy as np
import pytest
import torch

from conftest import golden

pytestmark = pytest.mark.gpu

SETTINGS = {"compression": "fri", "sampling_method": "systematic", "verbose": False,
            "compressed_contractions": ["O^2V^4", "O^3V^3", "O^4V^2"]}


def _golden_system():
    from fricc_gb300.synthetic import SyntheticSystem
    g = golden("iteration.npz")
    s = SyntheticSystem.__new__(SyntheticSystem)
    s.nocc, s.L, s.mo_energy = int(g["nocc"]), g["L"], g["mo_energy"]
    s.naux, s.nvir = s.L.shape[0], s.mo_energy.size - int(g["nocc"])
    s.sigma, s.seed = 0.0, 0
    return g, s


def _solver(system, m, precision="fp64"):
    from fricc_gb300.rccsd_dense import DeviceERIs
    from fricc_gb300.friccsd import FRICCSDGPU
    E = DeviceERIs.from_system(system)
    return FRICCSDGPU(E, dict(SETTINGS, m_keep=m), precision=precision)


def _oracle_step(eris, m, t1, t2, rn):
    from oracle import ccsd_oracle as CO
    draws = iter(rn)
    return CO.update_amps(dict(SETTINGS, m_keep=m), t1, t2, eris, rn_draw=lambda: next(draws))


def test_golden_iterates_teacher_forced(gpulib, oracle):
    from oracle import pyscf_standin as P
    g, s = _golden_system()
    m = int(g["m"])
    gs = _solver(s, m)
    eris = P.make_eris(s)
    rn = list(g["rn"])
    for it in range(len(g["energies"])):
        t1 = torch.from_numpy(g["t1"][it]).cuda()
        t2 = torch.from_numpy(g["t2"][it]).cuda()
        t1n, t2n = gs.update_amps(t1, t2, rn=rn[2 * it: 2 * it + 2])
        e, _ = gs.read_energy()
        assert abs(e - g["energies"][it]) < 1e-10, (it, e, g["energies"][it])
        scale = np.abs(g["t2"][it + 1]).max()
        assert np.abs(t2n.cpu().numpy() - g["t2"][it + 1]).max() < 1e-12 * scale
        e_or = P.ccsd_energy(*_oracle_step(eris, m, g["t1"][it], g["t2"][it], rn[2 * it: 2 * it + 2]), eris)
        assert abs(e - e_or) < 1e-10


@pytest.mark.parametrize("seed,precision", [(0, "fp64"), (1, "fp64"), (0, "df64"), (2, "df64")])
def test_o10v40_teacher_forced(gpulib, oracle, seed, precision):
    """The o10v40 workload (m = 20000): five steps along the GPU trajectory,
    with the sparse terms in FP64 or in FP32-pair arithmetic."""
    from oracle import pyscf_standin as P
    from fricc_gb300.synthetic import SyntheticSystem
    s = SyntheticSystem(10, 40, 200, 0.05, seed)
    m = 20000
    gs = _solver(s, m, precision)
    eris = P.make_eris(s)
    t1h, t2h = s.mp2_amplitudes()
    rng = np.random.default_rng(seed)
    t1, t2 = torch.from_numpy(t1h).cuda(), torch.from_numpy(t2h).cuda()
    for it in range(5):
        rn = [float(rng.random()), float(rng.random())]
        t1_in, t2_in = t1.cpu().numpy(), t2.cpu().numpy()
        t1, t2 = gs.update_amps(t1, t2, rn=rn)
        e_gpu, normt = gs.read_energy()
        o1, o2 = _oracle_step(eris, m, t1_in, t2_in, rn)
        e_or = P.ccsd_energy(o1, o2, eris)
        assert abs(e_gpu - e_or) < 1e-10, (it, e_gpu, e_or)
        g2 = t2.cpu().numpy()
        assert np.abs(g2 - o2).max() < 1e-12 * np.abs(o2).max()
        nref = np.linalg.norm(P.amplitudes_to_vector(o1, o2) - P.amplitudes_to_vector(t1_in, t2_in))
        assert abs(normt - nref) < 1e-10 * max(nref, 1.0)


def test_o10v40_free_running(gpulib, oracle):
    """Twenty iterations from MP2 with the same draws on both sides."""
    from oracle import ccsd_oracle as CO
    from oracle import pyscf_standin as P
    from fricc_gb300.synthetic import SyntheticSystem
    s = SyntheticSystem(10, 40, 200, 0.05, 0)
    m = 20000
    rng = np.random.default_rng(123)
    draws = [float(v) for v in rng.random(40)]
    gs = _solver(s, m)
    it_draws = iter(draws)
    gs.rn_draw = lambda: next(it_draws)
    t1h, t2h = s.mp2_amplitudes()
    conv, e, t1, t2, eg = gs.kernel(torch.from_numpy(t1h).cuda(), torch.from_numpy(t2h).cuda(), max_cycle=20,
                                   tol=0.0, tolnormt=0.0)
    od = iter(draws)
    conv, e, _, _, eo = CO.kernel(dict(SETTINGS, m_keep=m), P.make_eris(s), t1h, t2h, max_cycle=20, tol=0.0,
                                  tolnormt=0.0, rn_draw=lambda: next(od))
    diff = np.abs(np.array(eg) - np.array(eo))
    # the same sample path gives rounding-level agreement; report the whole trajectory
    print("max |dE| over 20 iterations:", diff.max())
    assert diff[:5].max() < 1e-10
    assert diff.max() < 1e-6


def test_e2e_host_entry(gpulib):
    from fricc_gb300.synthetic import SyntheticSystem
    s = SyntheticSystem(6, 20, 100, 0.05, 2)
    gs = _solver(s, 3000)
    t1h, t2h = s.mp2_amplitudes()
    a1, a2 = gs.update_amps_host(t1h, t2h, rn=[0.1, 0.2])
    b1, b2 = gs.update_amps(torch.from_numpy(t1h).cuda(), torch.from_numpy(t2h).cuda(), rn=[0.1, 0.2])
    assert np.array_equal(a2, b2.cpu().numpy()) and np.array_equal(a1, b1.cpu().numpy())


@pytest.mark.parametrize("precision", ["fp64", "df64"])
def test_unbiased_golden_teacher_forced(gpulib, precision):
    """The running-average W compression after burn-in against the reference's
    own trajectory (tests/golden/unbiased.npz): the average of the inputs is
    bit for bit numpy's, so every compression matches and each step's energy
    agrees to 1e-10 Eh."""
    from fricc_gb300.friccsd import FRICCSDGPU
    from fricc_gb300.rccsd_dense import DeviceERIs
    from fricc_gb300.synthetic import SyntheticSystem
    g = golden("unbiased.npz")
    s = SyntheticSystem.__new__(SyntheticSystem)
    s.nocc, s.L, s.mo_energy = int(g["nocc"]), g["L"], g["mo_energy"]
    s.naux, s.nvir = s.L.shape[0], s.mo_energy.size - int(g["nocc"])
    s.sigma, s.seed = 0.0, 0
    b = int(g["burn_in"])
    gs = FRICCSDGPU(DeviceERIs.from_system(s), dict(SETTINGS, m_keep=int(g["m"]), unbiased=True, burn_in=b),
                    precision=precision)
    rn = list(g["rn"])
    y = None
    for it in range(len(g["energies"])):
        t1 = torch.from_numpy(g["t1"][it]).cuda()
        t2 = torch.from_numpy(g["t2"][it]).cuda()
        t1n, t2n = gs.update_amps(t1, t2, rn=rn[2 * it: 2 * it + 2])
        e, _ = gs.read_energy()
        assert abs(e - g["energies"][it]) < 1e-10, (it, e, g["energies"][it])
        ref = g["t2"][it + 1]
        assert np.abs(t2n.cpu().numpy() - ref).max() < 1e-10 * np.abs(ref).max()
        if it >= b:
            k = it - b
            y = g["t2"][it] if k <= 1 else g["t2"][it] / k + (k - 1) / k * y
            assert np.array_equal(gs._t2_avg.cpu().numpy(), y), it
    assert y is not None
