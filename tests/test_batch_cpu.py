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


def test_server_admission_respects_hbm_budget(monkeypatch):
    """The request server's dispatcher admits a request only while the
    estimated footprints in flight fit the budget (a request larger than the
    budget runs alone), and every request finishes (solves faked on CPU)."""
    import threading
    import time

    from fricc_gb300 import batch as B
    monkeypatch.setattr(B.torch.cuda, "set_device", lambda d: None)
    monkeypatch.setattr(B.torch.cuda, "Stream", lambda device=None: object())
    lock = threading.Lock()
    state = {"in_use": 0, "max": 0, "n": 0}

    def fake_solve(self, req, t0, stream):
        need = B.footprint_bytes(req.nocc, req.nvir, self.precision)
        with lock:
            state["in_use"] += need
            state["max"] = max(state["max"], state["in_use"])
            state["n"] += 1
        req.started = time.perf_counter() - t0
        time.sleep(0.005 * (1 + req.rid % 3))
        req.energies, req.iterations, req.converged, req.e_corr = [-1.0], 1, True, -1.0
        with lock:
            state["in_use"] -= need

    monkeypatch.setattr(B.SolveServer, "_solve", fake_solve)
    reqs = request_stream(16, rate=1000.0, seed=3, nocc=(5, 12))
    sizes = sorted(B.footprint_bytes(r.nocc, r.nvir, "split") for r in reqs)
    budget = sizes[-1] + sizes[-2] // 2   # the two largest never run together
    srv = B.SolveServer(n_workers=4, hbm_budget=budget, precision="split", device="cuda:0")
    out = srv.run(reqs, time_scale=0.0)
    assert state["n"] == 16 and all(r.finished >= r.admitted >= 0 for r in out)
    assert state["max"] <= budget
    s = latency_summary(out)
    assert s["n"] == 16 and s["converged"] == 16 and s["solves_per_s"] > 0


def test_iteration_scheduler_interleaves_requests(monkeypatch):
    """schedule="iterations": builder threads build each request and issue
    its first iteration; one scheduler thread issues every later iteration,
    a request's next one only after its last one finished, with the
    iterations of different requests interleaved; the active-request cap
    and the HBM budget hold, and every request finishes (device work faked
    on CPU: an iteration "finishes" a few milliseconds after it is issued)."""
    import threading
    import time

    from fricc_gb300 import batch as B
    monkeypatch.setattr(B.torch.cuda, "set_device", lambda d: None)
    lock = threading.Lock()
    log = []            # (thread name, rid, iteration) of every issue
    state = {"live": 0, "max_live": 0, "in_use": 0, "max_in_use": 0}

    class FakeEvent:
        def __init__(self, ready_at):
            self.ready_at = ready_at

        def query(self):
            return time.perf_counter() >= self.ready_at

    class FakeOwn:
        stream = None

    def fake_build(self, req, t0, stream):
        need = B.footprint_bytes(req.nocc, req.nvir, self.precision)
        with lock:
            state["live"] += 1
            state["max_live"] = max(state["max_live"], state["live"])
            state["in_use"] += need
            state["max_in_use"] = max(state["max_in_use"], state["in_use"])
        req.started = time.perf_counter() - t0
        return B._Live(req, object(), None, stream, None, None, 0.0, time.perf_counter())

    def fake_issue(self, lv):
        with lock:
            log.append((threading.current_thread().name, lv.req.rid, lv.req.iterations))
        assert lv.event is None or lv.event.query()  # never ahead of the last iteration
        lv.event = FakeEvent(time.perf_counter() + 0.002 * (1 + lv.req.rid % 3))

    def fake_settle(self, lv):
        lv.req.iterations += 1
        lv.req.energies.append(-1.0 / lv.req.iterations)
        done = lv.req.iterations >= 3 + lv.req.rid % 2
        lv.req.converged = done
        return done

    def fake_close(self, lv):
        req = lv.req
        req.e_corr = req.energies[-1]
        with lock:
            state["live"] -= 1
            state["in_use"] -= B.footprint_bytes(req.nocc, req.nvir, self.precision)
        lv.solver = None

    monkeypatch.setattr(B.SolveServer, "_build", fake_build)
    monkeypatch.setattr(B.SolveServer, "_issue", fake_issue)
    monkeypatch.setattr(B.SolveServer, "_settle", fake_settle)
    monkeypatch.setattr(B.SolveServer, "_close", fake_close)
    monkeypatch.setattr(B.SolveServer, "_take_stream", lambda self: FakeOwn())
    reqs = request_stream(20, rate=2000.0, seed=4, nocc=(5, 12))
    sizes = sorted(B.footprint_bytes(r.nocc, r.nvir, "split") for r in reqs)
    budget = sum(sizes[-3:])
    srv = B.SolveServer(precision="split", device="cuda:0", schedule="iterations", max_active=5, n_builders=2,
                        hbm_budget=budget)
    out = srv.run(reqs, time_scale=0.0)
    assert all(r.iterations == 3 + r.rid % 2 and r.converged and r.finished >= r.started >= 0 for r in out)
    assert state["max_live"] <= 5 and state["max_in_use"] <= budget and state["live"] == 0
    first = {}
    later_threads = set()
    for name, rid, it in log:
        if it == 0:
            first[rid] = name
        else:
            later_threads.add(name)
    assert len(first) == 20 and len(later_threads) == 1   # one scheduler issues every later iteration
    assert not set(first.values()) & later_threads          # first iterations come from the builders
    later = [rid for _, rid, it in log if it > 0]
    switches = sum(a != b for a, b in zip(later, later[1:]))
    assert switches > len(set(later))                        # requests' iterations interleave


def test_iteration_scheduler_failure_releases_every_request(monkeypatch):
    """A failure inside the scheduler's own loop (here: the event query of a
    request's iteration raises, as it would after a device error) ends the
    run with that error instead of leaving the dispatcher waiting for HBM
    that no request gives back (device work faked on CPU)."""
    import time

    from fricc_gb300 import batch as B
    monkeypatch.setattr(B.torch.cuda, "set_device", lambda d: None)

    class BadEvent:
        def query(self):
            raise RuntimeError("device error seen by the event query")

    class FakeOwn:
        stream = None

    def fake_build(self, req, t0, stream):
        req.started = time.perf_counter() - t0
        return B._Live(req, object(), None, stream, None, None, 0.0, time.perf_counter())

    def fake_issue(self, lv):
        lv.event = BadEvent()

    monkeypatch.setattr(B.SolveServer, "_build", fake_build)
    monkeypatch.setattr(B.SolveServer, "_issue", fake_issue)
    monkeypatch.setattr(B.SolveServer, "_take_stream", lambda self: FakeOwn())
    reqs = request_stream(12, rate=5000.0, seed=2, nocc=(5, 8))
    budget = 3 * max(B.footprint_bytes(r.nocc, r.nvir, "split") for r in reqs)
    srv = B.SolveServer(precision="split", device="cuda:0", schedule="iterations", max_active=2, n_builders=2,
                        hbm_budget=budget)
    import pytest
    with pytest.raises(RuntimeError, match="device error"):
        srv.run(reqs, time_scale=0.0)
    assert srv._in_use == 0 and srv._n_live == 0
