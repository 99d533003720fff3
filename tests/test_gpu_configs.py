"""The configurations at their own sizes.

* Split precision at nocc=40, nvir=200 (naux=1200, m = 5% of o^2 v^2 =
  3.2M): two teacher-forced steps of the split form against the FP64 GPU
  path from the same amplitudes and draws -- |dE_corr| <= 1e-6 Eh per step,
  and both forms compress bit for bit alike.
* Batched replicas at nocc=20, nvir=100 (naux=600, m = 5% = 200,000): one
  batch step of 16 replicas with distinct seeds, each replica equal to its
  lone solve.

The synthetic systems are the workloads' own generator (factor entries
N(0, sigma^2 / naux))."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _export(handle, m):
    from fricc_gb300 import _lib as L
    flat = np.empty(m, dtype=np.int64)
    vals = np.empty(m, dtype=np.float64)
    L.check(L.load().fricc_sp_export(handle, ctypes.c_void_p(flat.ctypes.data), ctypes.c_void_p(vals.ctypes.data),
                                     ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return flat, vals


def test_split_o40v200_two_steps_vs_fp64(gpulib):
    from fricc_gb300.batch import mp2_device
    from fricc_gb300.cholesky import split_eris
    from fricc_gb300.friccsd import FRICCSDGPU
    from fricc_gb300.rccsd_dense import DeviceERIs
    from fricc_gb300.synthetic import WORKLOADS, make_system
    w = WORKLOADS["o40v200"]
    m = w["m"]
    assert (w["nocc"], w["nvir"], w["naux"], m) == (40, 200, 1200, 3_200_000)
    system = make_system("o40v200", seed=0)
    E = DeviceERIs.from_system(system)
    Es = split_eris(system)
    ref = FRICCSDGPU(E, {"m_keep": m}, precision="fp64")
    spl = FRICCSDGPU(Es, {"m_keep": m}, precision="split")
    t1, t2 = mp2_device(E)
    draws = [(0.8401877171547095, 0.3943829268190930), (0.7830992237586059, 0.7984400334760733)]
    for step, rn in enumerate(draws):
        r1, r2 = ref.update_amps(t1, t2, rn=list(rn))
        e_ref = ref.read_energy()[0]
        spl.update_amps(t1, t2, rn=list(rn))
        e_spl = spl.read_energy()[0]
        assert abs(e_spl - e_ref) <= 1e-6, (step, e_spl, e_ref)
        for h_ref, h_spl in ((ref._sp, spl._sp), (ref._sp_w, spl._sp_w)):
            fr, vr = _export(h_ref.h, m)
            fs, vs = _export(h_spl.h, m)
            assert np.array_equal(fr, fs) and np.array_equal(vr.view(np.int64), vs.view(np.int64)), step
        t1, t2 = r1, r2   # teacher forcing: both forms continue from the FP64 iterate
    del ref, spl, E, Es
    torch.cuda.empty_cache()


def test_batch_o20v100_sixteen_replicas_equal_their_lone_solves(gpulib):
    from fricc_gb300.batch import ReplicaBatch, mp2_device
    from fricc_gb300.friccsd import FRICCSDGPU
    from fricc_gb300.rccsd_dense import DeviceERIs
    from fricc_gb300.rng import GlibcRand
    from fricc_gb300.synthetic import WORKLOADS, make_system
    w = WORKLOADS["o20v100x64"]
    m = w["m"]
    assert (w["nocc"], w["nvir"], w["naux"], m) == (20, 100, 600, 200_000)
    E = DeviceERIs.from_system(make_system("o20v100x64", seed=0))
    seeds = list(range(100, 116))
    batch = ReplicaBatch(E, {"m_keep": m}, seeds, n_streams=8, precision="fp64")
    batch.step()
    for r, seed in enumerate(seeds):
        lone = FRICCSDGPU(E, {"m_keep": m}, rn_draw=GlibcRand(seed), precision="fp64")
        t1, t2 = mp2_device(E)
        t1, t2 = lone.update_amps(t1, t2)
        e = lone.read_energy()[0]
        assert abs(e - batch.history[r][0]) <= 1e-12 * max(1.0, abs(e)), (r, e, batch.history[r][0])
        torch.testing.assert_close(t2, batch.t2[r], rtol=1e-13, atol=1e-18)
    mean, var = batch.stats()
    assert np.isfinite(mean) and var > 0.0
