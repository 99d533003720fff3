"""The synthetic systems (fricc_gb300/synthetic.py): the named workloads'
sizes and the recipe's properties -- energy ranges, a symmetric factor with
entries N(0, sigma^2/naux), integrals with their permutational symmetry, MP2
amplitudes with t_ijab = t_jiba -- on the host and, for DeviceSystem, with
torch's generator on the CPU (the same code the GPU runs)."""
import numpy as np
import pytest
import torch

from fricc_gb300.synthetic import WORKLOADS, DeviceSystem, SyntheticSystem, make_system


def test_named_workloads():
    want = {"o10v40": (10, 40, 200, 0.05, 20000, 20), "o30v150": (30, 150, 900, 0.03, 2_000_000, 30),
            "o20v100x64": (20, 100, 600, 0.04, 200_000, 30), "o40v200": (40, 200, 1200, 0.025, 3_200_000, 40)}
    for name, (o, v, naux, sigma, m, iters) in want.items():
        w = WORKLOADS[name]
        assert (w["nocc"], w["nvir"], w["naux"], w["sigma"], w["m"], w["iters"]) == (o, v, naux, sigma, m, iters)
        assert m <= o * o * v * v
    assert WORKLOADS["o20v100x64"]["replicas"] == 64
    # m = 5% of N for the replica and largest workloads
    for name in ("o20v100x64", "o40v200"):
        w = WORKLOADS[name]
        assert w["m"] == w["nocc"] ** 2 * w["nvir"] ** 2 // 20


def _check_recipe(eo, ev, L, sigma, naux):
    assert np.all(np.diff(eo) >= 0) and np.all(np.diff(ev) >= 0)
    assert eo.min() >= -1.5 and eo.max() <= -0.3 and ev.min() >= 0.2 and ev.max() <= 3.0
    assert np.array_equal(L, L.transpose(0, 2, 1))
    iu = np.triu_indices(L.shape[1])
    x = L[:, iu[0], iu[1]].ravel()
    assert abs(x.mean()) < 5 * sigma / naux ** 0.5 / x.size ** 0.5
    assert x.std() == pytest.approx(sigma / naux ** 0.5, rel=0.05)


def test_host_system_recipe():
    s = SyntheticSystem(6, 20, 80, 0.05, seed=3)
    o = s.nocc
    _check_recipe(s.mo_energy[:o], s.mo_energy[o:], s.L, 0.05, 80)
    assert np.array_equal(s.fock, np.diag(s.mo_energy))
    ovov = s.eri("ovov")
    np.testing.assert_allclose(ovov, ovov.transpose(2, 3, 0, 1), rtol=0, atol=1e-15)
    np.testing.assert_allclose(s.eri("ovvo"), ovov.transpose(0, 1, 3, 2), rtol=0, atol=1e-15)
    t1, t2 = s.mp2_amplitudes()
    assert not t1.any() and t2.shape == (o, o, s.nvir, s.nvir) and t2.flags.c_contiguous
    np.testing.assert_allclose(t2, t2.transpose(1, 0, 3, 2), rtol=0, atol=1e-15)
    eia = s.mo_energy[:o, None] - s.mo_energy[None, o:]
    np.testing.assert_allclose(t2 * (eia[:, None, :, None] + eia[None, :, None, :]), ovov.transpose(0, 2, 1, 3),
                               rtol=1e-13, atol=1e-17)
    # seeded: the same seed gives the same system, another seed another
    assert np.array_equal(SyntheticSystem(6, 20, 80, 0.05, seed=3).L, s.L)
    assert not np.array_equal(SyntheticSystem(6, 20, 80, 0.05, seed=4).L, s.L)


def test_device_system_recipe_on_cpu():
    d = DeviceSystem(6, 20, 80, 0.05, seed=3, device="cpu")
    o = d.nocc
    e = d.mo_energy.numpy()
    _check_recipe(e[:o], e[o:], d.L.numpy(), 0.05, 80)
    assert torch.equal(d.fock, torch.diag(d.mo_energy))
    assert torch.equal(DeviceSystem(6, 20, 80, 0.05, seed=3, device="cpu").L, d.L)


def test_make_system_sizes():
    s = make_system("o10v40", seed=1)
    assert (s.nocc, s.nvir, s.naux, s.sigma, s.seed) == (10, 40, 200, 0.05, 1)
    assert s.L.shape == (200, 50, 50)
