"""Many FRI-CCSD solves on one GPU at once: replicas and served requests.

* ``ReplicaBatch`` -- independent FRI replicas of one system (distinct seeds)
  sharing the integrals in HBM; every replica keeps its own amplitudes, its
  two compressed-T2 handles and its own copy of the reference's libc random
  stream (``GlibcRand``), so each replica's trajectory is exactly the one a
  lone run with that seed gives.  One ``step()`` advances every replica by
  one iteration; replicas are spread over a pool of CUDA streams driven by
  host threads, so their kernels overlap on the device.
* ``SolveServer`` -- a request loop for solves of different (nocc, nvir):
  requests arrive over time, are admitted while their estimated HBM footprint
  fits a budget, keep their state resident while they iterate, and run
  concurrently on the stream pool; it records arrival, admission, start and
  finish times for latency percentiles and solves/s.

Host threads release the GIL inside every CUDA-library call and inside
torch's kernels, so the pool keeps several solves' work in flight.
"""
from __future__ import annotations

import math
import queue
import threading
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from .friccsd import FRICCSDGPU
from .rccsd_dense import DeviceERIs
from .rng import GlibcRand
from .synthetic import DeviceSystem, SyntheticSystem


def mp2_device(E: DeviceERIs):
    o = E.nocc
    e = E.mo_energy
    eia = e[:o, None] - e[None, o:]
    t2 = (E.ovov.permute(0, 2, 1, 3) / (eia[:, None, :, None] + eia[None, :, None, :])).contiguous()
    t1 = torch.zeros(o, e.numel() - o, dtype=torch.float64, device=E.device)
    return t1, t2


class ReplicaBatch:
    def __init__(self, eris: DeviceERIs, settings: dict, seeds, n_streams: int = 8, precision: str = "df64",
                 graph: bool = False):
        self.eris = eris
        self.seeds = list(seeds)
        self.n = len(self.seeds)
        # split precision: the replicas share one (vv|vv) operand, rebuilt once
        self.solvers = [FRICCSDGPU(eris, settings, rn_draw=GlibcRand(s), precision=precision, graph=graph,
                                   rebuild_vvvv=precision != "split")
                        for s in self.seeds]
        t1, t2 = mp2_device(eris)
        self.t1 = [t1.clone() for _ in range(self.n)]
        self.t2 = [t2.clone() for _ in range(self.n)]
        self.k = max(1, min(n_streams, self.n))
        self.streams = [torch.cuda.Stream(device=eris.device) for _ in range(self.k)]
        self.history = [[] for _ in range(self.n)]
        self._errors = []
        self._dev = eris.device.index if eris.device.index is not None else torch.cuda.current_device()
        torch.cuda.current_stream().synchronize()  # the clones above must land before other streams read them

    def _work(self, w):
        try:
            torch.cuda.set_device(self._dev)
            with torch.cuda.stream(self.streams[w]):
                for r in range(w, self.n, self.k):
                    self.t1[r], self.t2[r] = self.solvers[r].update_amps(self.t1[r], self.t2[r])
        except BaseException as e:  # surfaced by step()
            self._errors.append(e)

    def _capture_batch(self):
        """One CUDA graph for an iteration of every replica: each replica's
        iteration is captured on a stream of its own (forked from the capture
        stream and joined back), reading static amplitudes and device-resident
        draws and writing the new amplitudes back into the static inputs, so
        each replay advances the whole batch by one iteration."""
        from . import _lib as L
        from .friccsd import _CAPTURE_LOCK
        dev = self.eris.device
        self._bt1 = [t.contiguous().clone() for t in self.t1]
        self._bt2 = [t.contiguous().clone() for t in self.t2]
        self._brn = torch.zeros(self.n, 2, dtype=torch.float64, device=dev)
        self._bstreams = [L.OwnStream(dev) for _ in range(self.n)]
        self._bcap = L.OwnStream(dev)
        cs, cur = self._bcap.stream, torch.cuda.current_stream()
        g = torch.cuda.CUDAGraph()
        with _CAPTURE_LOCK:
            cs.wait_stream(cur)
            with torch.cuda.stream(cs):
                g.capture_begin(capture_error_mode="thread_local")
                try:
                    for r, sol in enumerate(self.solvers):
                        sr = self._bstreams[r].stream
                        sr.wait_stream(cs)
                        with torch.cuda.stream(sr):
                            o1, o2 = sol._update_eager(self._bt1[r], self._bt2[r], rn_dev=self._brn[r])
                            self._bt1[r].copy_(o1)
                            self._bt2[r].copy_(o2)
                        cs.wait_stream(sr)
                finally:
                    g.capture_end()
            cur.wait_stream(cs)
        self._bgraph = g

    def step_graph(self, record: bool = True):
        """One iteration of every replica as one replay of the batch graph
        (captured at the first call; the replicas' handles must exist, i.e.
        one eager ``step()`` first)."""
        if getattr(self, "_bgraph", None) is None:
            self._capture_batch()
        draws = [[sol.rn_draw(), sol.rn_draw()] for sol in self.solvers]  # the reference's order per replica
        self._brn.copy_(torch.tensor(draws, dtype=torch.float64))
        self._bgraph.replay()
        for sol in self.solvers:
            sol._iter += 1
        self.t1, self.t2 = self._bt1, self._bt2
        torch.cuda.current_stream().synchronize()
        if record:
            for r in range(self.n):
                self.history[r].append(self.solvers[r].read_energy()[0])

    def step(self, record: bool = True):
        """One iteration of every replica (all streams joined on return)."""
        threads = [threading.Thread(target=self._work, args=(w,)) for w in range(self.k)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        if self._errors:
            raise self._errors[0]
        for s in self.streams:
            s.synchronize()
        if record:
            for r in range(self.n):
                self.history[r].append(self.solvers[r].read_energy()[0])

    def energies(self) -> np.ndarray:
        return np.array([h[-1] for h in self.history])

    def stats(self):
        e = self.energies()
        return float(e.mean()), float(e.var(ddof=1)) if e.size > 1 else 0.0

    def trace_stats(self, burn: int = 0):
        """Error bars of the time-averaged energy of each replica's trace
        after ``burn`` iterations, as fri-cc's ``mcmc_std`` gives them
        (sqrt(tau / n var), tau the integrated autocorrelation time; a trace
        too short for a reliable tau warns instead of raising).  Returns
        (means, error bars, taus), one entry per replica."""
        from .stats import mcmc_std
        means, errs, taus = [], [], []
        for h in self.history:
            x = np.asarray(h[burn:], dtype=np.float64)
            err, tau = mcmc_std(x, quiet=True)
            means.append(float(x.mean()))
            errs.append(float(err))
            taus.append(float(tau))
        return np.array(means), np.array(errs), np.array(taus)


# ---------------------------------------------------------------------------
@dataclass
class Request:
    rid: int
    arrival: float           # seconds after the stream starts
    nocc: int
    nvir: int
    naux: int
    frac: float              # kept fraction of o^2 v^2
    seed: int
    sigma: float = 0.05
    # filled in by the server
    admitted: float = math.nan
    started: float = math.nan
    finished: float = math.nan
    iterations: int = 0
    build_s: float = math.nan    # system, integrals, solver and MP2 guess (stream-synchronised)
    iterate_s: float = math.nan  # the iterations to convergence
    converged: bool = False
    e_corr: float = math.nan
    energies: list = field(default_factory=list)

    @property
    def m(self):
        return max(1, int(self.frac * self.nocc * self.nocc * self.nvir * self.nvir))


def request_stream(n: int, rate: float, seed: int = 0, nocc=(5, 30), ratio=(4.0, 6.0), frac=(0.05, 0.20)):
    """Poisson arrivals; nocc ~ U{lo..hi}, nvir = ceil(r nocc) with r ~ U[ratio],
    naux = 8 (nocc + nvir), kept fraction ~ U[frac], a seed per request."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        o = int(rng.integers(nocc[0], nocc[1] + 1))
        v = int(math.ceil(rng.uniform(*ratio) * o))
        out.append(Request(i, t, o, v, 8 * (o + v), float(rng.uniform(*frac)), int(rng.integers(1, 2**31 - 1))))
    return out


def footprint_bytes(o: int, v: int, precision: str = "df64") -> int:
    """HBM a resident solve needs: integral blocks and the layouts derived from
    them (vvvv and its float-pair form, ovvv in nine layouts or forms),
    amplitudes and work arrays (~16 o^2v^2).  Split precision keeps (vv|vv)
    only as the FP32 block it rebuilds (v^4 / 2 doubles) and adds the
    BF16x3 operand splits (~4.5 o v^3 doubles)."""
    vvvv = 0.5 * v**4 if precision == "split" else 2 * v**4
    ovvv = 13.5 * o * v**3 if precision == "split" else 9 * o * v**3
    return int(8 * (vvvv + ovvv + 16 * o * o * v * v + 4 * o**4 + 8 * o**3 * v))


class _Live:
    """A served request between its build and its last iteration: its
    solver, amplitudes and stream, the energy it compares the next one
    with, and the event its iteration in flight records."""

    __slots__ = ("req", "solver", "E", "stream", "t1", "t2", "eold", "event", "ti", "owner")

    def __init__(self, req, solver, E, stream, t1, t2, eold, ti):
        self.req, self.solver, self.E, self.stream = req, solver, E, stream
        self.t1, self.t2, self.eold, self.ti = t1, t2, eold, ti
        self.event = None
        self.owner = None


class SolveServer:
    """Serve solve requests on one GPU.

    schedule="iterations" (continuous batching at iteration level): builder
    threads make each admitted request's system, integrals, solver and first
    iteration on a stream of the request's own; one scheduler thread then
    drives every built request an iteration at a time, issuing a request's
    next iteration as soon as its last one has finished on the device
    (polled through an event), so the iterations of all requests in flight
    overlap on the GPU while one host thread issues them -- requests join
    and leave between iterations as they are built and converge.
    schedule="workers": n_workers threads each solve one request at a time
    from build to convergence (several host threads issuing at once contend
    for the interpreter lock, which measured slower than one issuing thread).
    """

    def __init__(self, n_workers: int = 8, hbm_budget: float = 200e9, precision: str = "df64", max_cycle: int = 30,
                 tol: float = 1e-7, device="cuda", graph: bool = False, device_inputs: bool = True,
                 rebuild_vvvv: bool = True, schedule: str = "workers", max_active: int = 24, n_builders: int = 2):
        if schedule not in ("workers", "iterations"):
            raise ValueError("schedule must be 'workers' or 'iterations'")
        self.schedule = schedule
        self.max_active = max(1, int(max_active))
        self.n_builders = max(1, int(n_builders))
        self.graph = graph
        # split precision: rebuild (vv|vv) every iteration, or once per solve
        self.rebuild_vvvv = rebuild_vvvv
        # draw each request's synthetic system on the GPU (DeviceSystem) or
        # on the host (SyntheticSystem, numpy)
        self.device_inputs = device_inputs
        self.k = n_workers
        self.budget = hbm_budget
        self.precision = precision
        self.max_cycle = max_cycle
        self.tol = tol
        self.device = torch.device(device)
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        self._in_use = 0
        self._n_live = 0
        self._cv = threading.Condition()
        self._streams = []  # idle streams of finished requests, reused

    def _take_stream(self):
        """A stream of the request's own (created for it, not torch's shared
        pool, whose few streams would tie requests together)."""
        with self._cv:
            if self._streams:
                return self._streams.pop()
        from ._lib import OwnStream
        return OwnStream(self.device)

    def _give_stream(self, own) -> None:
        with self._cv:
            self._streams.append(own)

    # ------------------------------------------------------------ one request
    def _build(self, req: Request, t0: float, stream) -> _Live:
        """System, integrals, solver and MP2 guess of a request on ``stream``
        (waited for: build_s is its time)."""
        tb = time.perf_counter()
        with torch.cuda.stream(stream):
            if self.device_inputs:
                system = DeviceSystem(req.nocc, req.nvir, req.naux, req.sigma, req.seed, device=self.device)
            else:
                system = SyntheticSystem(req.nocc, req.nvir, req.naux, req.sigma, req.seed)
            if self.precision == "split":  # integrals rebuilt from the BF16 hi+lo factor on the tensor cores
                from .cholesky import split_eris
                E = split_eris(system, device=self.device)
            else:
                E = DeviceERIs.from_system(system, device=self.device)
            solver = FRICCSDGPU(E, {"m_keep": req.m}, rn_draw=GlibcRand(req.seed), precision=self.precision,
                                graph=self.graph, rebuild_vvvv=self.rebuild_vvvv)
            t1, t2 = mp2_device(E)
            stream.synchronize()
            ti = time.perf_counter()
            req.started = ti - t0
            req.build_s = ti - tb
            eold = solver.energy(t1, t2)
        return _Live(req, solver, E, stream, t1, t2, eold, ti)

    def _issue(self, lv: _Live) -> None:
        """Launch the request's next iteration; its event marks the end."""
        with torch.cuda.stream(lv.stream):
            lv.t1, lv.t2 = lv.solver.update_amps(lv.t1, lv.t2)
            ev = torch.cuda.Event()
            ev.record(lv.stream)
        lv.event = ev

    def _settle(self, lv: _Live) -> bool:
        """Read the finished iteration's energy; True when the request is
        done (converged, diverged or out of iterations)."""
        req = lv.req
        with torch.cuda.stream(lv.stream):
            e, _ = lv.solver.read_energy()
        req.energies.append(e)
        req.iterations += 1
        if abs(e - lv.eold) < self.tol:
            req.converged = True
            return True
        if not math.isfinite(e) or abs(e - lv.eold) > 1e5:
            return True
        lv.eold = e
        return req.iterations >= self.max_cycle

    def _close(self, lv: _Live) -> None:
        req = lv.req
        req.e_corr = req.energies[-1] if req.energies else math.nan
        lv.stream.synchronize()
        req.iterate_s = time.perf_counter() - lv.ti
        lv.solver = lv.E = lv.t1 = lv.t2 = lv.event = None

    def _solve(self, req: Request, t0: float, stream):
        lv = self._build(req, t0, stream)
        done = self.max_cycle <= 0
        while not done:
            self._issue(lv)
            done = self._settle(lv)
        self._close(lv)

    # ----------------------------------------------------------- the stream
    def _release(self, req: Request) -> None:
        with self._cv:
            self._in_use -= footprint_bytes(req.nocc, req.nvir, self.precision)
            self._n_live -= 1
            self._cv.notify_all()

    def run(self, requests, time_scale: float = 1.0):
        """Serve the requests (arrival times scaled by time_scale); returns them filled in."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        admitted = queue.Queue()
        t0 = time.perf_counter()
        errors = []
        iterations = self.schedule == "iterations"
        n_consumers = self.n_builders if iterations else self.k
        cap = self.max_active if iterations else 1 << 30

        def dispatcher():
            for r in reqs:
                delay = r.arrival * time_scale - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
                need = footprint_bytes(r.nocc, r.nvir, self.precision)
                with self._cv:
                    while (self._in_use + need > self.budget or self._n_live >= cap) and self._n_live > 0:
                        self._cv.wait()
                    self._in_use += need
                    self._n_live += 1
                r.admitted = time.perf_counter() - t0
                admitted.put(r)
            for _ in range(n_consumers):
                admitted.put(None)

        def worker(w):
            torch.cuda.set_device(self.device)
            stream = torch.cuda.Stream(device=self.device)
            while True:
                r = admitted.get()
                if r is None:
                    return
                try:
                    self._solve(r, t0, stream)
                except BaseException as e:
                    errors.append(e)
                r.finished = time.perf_counter() - t0
                self._release(r)

        built = queue.Queue()

        def builder(w):
            torch.cuda.set_device(self.device)
            try:
                while True:
                    r = admitted.get()
                    if r is None:
                        return
                    try:
                        own = self._take_stream()
                        lv = self._build(r, t0, own.stream)
                        lv.owner = own
                        if self.max_cycle > 0:
                            self._issue(lv)  # the first iteration (handles and first-use splits) here
                        built.put(lv)
                    except BaseException as e:
                        errors.append(e)
                        r.finished = time.perf_counter() - t0
                        self._release(r)
            finally:
                built.put(None)

        def scheduler():
            active = []
            open_builders = self.n_builders
            try:
                torch.cuda.set_device(self.device)
                while open_builders or active:
                    while True:  # requests built since the last pass join
                        try:
                            lv = built.get_nowait() if active or not open_builders else built.get(timeout=0.05)
                        except queue.Empty:
                            break
                        if lv is None:
                            open_builders -= 1
                        else:
                            active.append(lv)
                    progressed = False
                    for lv in list(active):
                        if lv.event is not None and not lv.event.query():
                            continue
                        progressed = True
                        try:
                            done = lv.event is None or self._settle(lv)
                            if not done:
                                self._issue(lv)
                                continue
                            self._close(lv)
                        except BaseException as e:
                            errors.append(e)
                        lv.req.finished = time.perf_counter() - t0
                        active.remove(lv)
                        if lv.solver is None:  # closed: its stream is idle
                            self._give_stream(lv.owner)
                        self._release(lv.req)
                    if active and not progressed:
                        time.sleep(2e-4)
            except BaseException as e:
                # the scheduler itself failed (e.g. a device error seen by an
                # event query): hand back every live request so that the
                # dispatcher and the builders run to their end
                errors.append(e)
                for lv in active:
                    lv.req.finished = time.perf_counter() - t0
                    self._release(lv.req)
                while open_builders:
                    lv = built.get()
                    if lv is None:
                        open_builders -= 1
                    else:
                        lv.req.finished = time.perf_counter() - t0
                        self._release(lv.req)

        if iterations:
            th = ([threading.Thread(target=dispatcher), threading.Thread(target=scheduler)]
                  + [threading.Thread(target=builder, args=(w,)) for w in range(self.n_builders)])
        else:
            th = [threading.Thread(target=dispatcher)] + [threading.Thread(target=worker, args=(w,))
                                                          for w in range(self.k)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        if errors:
            raise errors[0]
        return reqs


def latency_summary(reqs, time_scale=1.0):
    lat = np.array([r.finished - r.arrival * time_scale for r in reqs])
    span = max(r.finished for r in reqs) - min(r.arrival * time_scale for r in reqs)
    build = float(sum(r.build_s for r in reqs))
    iterate = float(sum(r.iterate_s for r in reqs))
    its = int(sum(r.iterations for r in reqs))
    return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "solves_per_s": len(reqs) / span, "iterations": its,
            "converged": int(sum(r.converged for r in reqs)), "n": len(reqs),
            # summed over requests (concurrent requests overlap, so these add
            # up to more than the span when several workers run)
            "build_s_sum": build, "iterate_s_sum": iterate, "build_share": build / max(build + iterate, 1e-30)}
