"""Batched replicas and served requests: every result is the same alone and in
the mix (same seed, same draws; kernels are deterministic, so the energies
agree to rounding: bound 1e-10 Eh, in practice bit for bit)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_replicas_alone_and_in_the_mix(gpulib):
    from fricc_gb300.batch import ReplicaBatch, mp2_device
    from fricc_gb300.friccsd import FRICCSDGPU
    from fricc_gb300.rccsd_dense import DeviceERIs
    from fricc_gb300.rng import GlibcRand
    from fricc_gb300.synthetic import SyntheticSystem
    s = SyntheticSystem(6, 24, 120, 0.05, 3)
    E = DeviceERIs.from_system(s)
    settings = {"m_keep": 4000}
    seeds = [11, 12, 13, 14, 15, 16, 17, 18, 19, 20, 21, 22]
    batch = ReplicaBatch(E, settings, seeds, n_streams=6, precision="df64")
    for _ in range(4):
        batch.step()
    for r, seed in enumerate(seeds):
        lone = FRICCSDGPU(E, settings, rn_draw=GlibcRand(seed), precision="df64")
        t1, t2 = mp2_device(E)
        hist = []
        for _ in range(4):
            t1, t2 = lone.update_amps(t1, t2)
            hist.append(lone.read_energy()[0])
        assert np.max(np.abs(np.array(hist) - np.array(batch.history[r]))) < 1e-10, (r, hist, batch.history[r])
    mean, var = batch.stats()
    assert np.isfinite(mean) and var > 0.0  # distinct seeds give distinct samples


@pytest.mark.parametrize("precision", ["df64", "split"])
def test_batch_graph_matches_eager(gpulib, precision):
    """One CUDA graph per batch step (every replica's iteration captured on
    its own stream) gives the trajectories of the eager batch."""
    from fricc_gb300.batch import ReplicaBatch
    from fricc_gb300.cholesky import split_eris
    from fricc_gb300.rccsd_dense import DeviceERIs
    from fricc_gb300.synthetic import SyntheticSystem
    s = SyntheticSystem(6, 24, 120, 0.05, 3)
    E = split_eris(s) if precision == "split" else DeviceERIs.from_system(s)
    settings = {"m_keep": 4000}
    seeds = [31, 32, 33, 34, 35]
    g = ReplicaBatch(E, settings, seeds, n_streams=3, precision=precision)
    e = ReplicaBatch(E, settings, seeds, n_streams=3, precision=precision)
    g.step()
    e.step()
    for _ in range(4):
        g.step_graph()
        e.step()
    for r in range(len(seeds)):
        assert np.max(np.abs(np.array(g.history[r]) - np.array(e.history[r]))) < 1e-13, r
    torch.testing.assert_close(g.t2[0], e.t2[0], rtol=1e-12, atol=1e-18)


@pytest.mark.parametrize("schedule", ["workers", "iterations"])
def test_served_requests_match_lone_solves(gpulib, schedule):
    from fricc_gb300.batch import SolveServer, request_stream
    reqs = request_stream(6, rate=200.0, seed=5, nocc=(4, 7))
    out = SolveServer(n_workers=3, precision="df64", max_cycle=4, schedule=schedule, max_active=4).run(reqs)
    for r in out:
        assert r.iterations >= 1 and np.isfinite(r.e_corr)
        assert r.admitted >= r.arrival - 1e-6 and r.finished >= r.started
    lone = request_stream(6, rate=200.0, seed=5, nocc=(4, 7))
    for r in lone:
        SolveServer(n_workers=1, precision="df64", max_cycle=4).run([r])
    for a, b in zip(sorted(out, key=lambda r: r.rid), sorted(lone, key=lambda r: r.rid)):
        assert abs(a.e_corr - b.e_corr) < 1e-10, (a.rid, a.e_corr, b.e_corr)


@pytest.mark.parametrize("schedule", ["workers", "iterations"])
def test_served_split_requests_alone_in_the_mix_and_against_fp64(gpulib, schedule):
    """The served split-precision form: each request's energies are the same
    served among others (3 workers, or the iteration-level scheduler with up
    to 4 requests in flight: overlapping solves) as solved alone, and every
    iteration's energy is within 1e-6 Eh of the plain FP64 GPU form's (same
    synthetic system, same draws)."""
    from fricc_gb300.batch import SolveServer, request_stream

    def stream():
        return request_stream(6, rate=200.0, seed=11, nocc=(5, 8))

    served = SolveServer(n_workers=3, precision="split", max_cycle=4, schedule=schedule, max_active=4).run(stream())
    lone, plain = stream(), stream()
    for r in lone:
        SolveServer(n_workers=1, precision="split", max_cycle=4).run([r])
    for r in plain:
        SolveServer(n_workers=1, precision="fp64", max_cycle=4).run([r])
    key = lambda r: r.rid  # noqa: E731
    for a, b, c in zip(sorted(served, key=key), sorted(lone, key=key), sorted(plain, key=key)):
        assert a.iterations == b.iterations >= 1 and np.isfinite(a.e_corr)
        assert np.max(np.abs(np.array(a.energies) - np.array(b.energies))) < 1e-10, a.rid
        n = min(len(a.energies), len(c.energies))
        assert np.max(np.abs(np.array(a.energies[:n]) - np.array(c.energies[:n]))) <= 1e-6, (a.rid, a.energies, c.energies)
