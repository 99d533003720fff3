"""Host logic of the request stream and the admission footprint (CPU)."""
import math

import numpy as np

from fricc_gb300.batch import footprint_bytes, latency_summary, request_stream


def test_request_stream_distribution():
    reqs = request_stream(2000, rate=50.0, seed=1)
    arr = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(arr) > 0)
    assert abs(len(reqs) / arr[-1] - 50.0) < 5.0
    for r in reqs:
        assert 5 <= r.nocc <= 30
        assert math.ceil(4 * r.nocc) <= r.nvir <= math.ceil(6 * r.nocc)
        assert r.naux == 8 * (r.nocc + r.nvir)
        assert 0.05 <= r.frac <= 0.20 and 1 <= r.m
    assert len({r.seed for r in reqs}) > 1990


def test_footprint_monotone_and_summary():
    assert footprint_bytes(30, 180) > footprint_bytes(10, 40) > footprint_bytes(5, 20) > 0
    reqs = request_stream(4, rate=10.0, seed=2)
    for k, r in enumerate(reqs):
        r.finished = r.arrival + 1.0 + k
        r.iterations = 3
    s = latency_summary(reqs)
    assert s["n"] == 4 and s["iterations"] == 12 and s["p50_s"] >= 1.0


def test_replica_trace_stats_is_mcmc_std():
    from fricc_gb300.batch import ReplicaBatch
    from fricc_gb300.stats import mcmc_std
    rng = np.random.default_rng(4)
    rb = ReplicaBatch.__new__(ReplicaBatch)  # only the recorded traces are needed
    rb.history = [list(-0.1 + 1e-4 * rng.standard_normal(400)) for _ in range(3)]
    means, errs, taus = rb.trace_stats(burn=50)
    for r in range(3):
        x = np.array(rb.history[r][50:])
        e, t = mcmc_std(x)
        assert means[r] == x.mean() and errs[r] == e and taus[r] == t
