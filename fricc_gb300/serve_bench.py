"""Throughput of the batched and served forms (python -m fricc_gb300.serve_bench).

  --mode replicas : R independent FRI replicas (distinct seeds) of the
                    o20v100 system (naux=600, m = 5% of o^2 v^2), all resident,
                    iterated together on a pool of streams (--fused: as one
                    stacked iteration, each kernel launched once for all
                    replicas); prints iterations/s
                    of the whole batch, the replica mean and variance of E_corr and
                    each replica's trace error bar (fri-cc's mcmc_std).
  --mode serve    : a Poisson stream of solve requests (nocc ~ U{5..30},
                    nvir = ceil(r nocc) with r ~ U[4,6], naux = 8(o+v), kept
                    fraction ~ U[5%,20%], converged at |dE| < 1e-7 Eh or
                    after --max-cycle iterations) served concurrently (by
                    default at iteration level: one scheduler thread issues
                    each request's next iteration when its last one is done),
                    against
                    the same requests solved one at a time in plain FP64;
                    prints solves/s and p50/p99 time to converged energy.
One JSON line per mode.
"""
from __future__ import annotations

import argparse
import json
import os
import time


def run_replicas(args):
    import numpy as np
    import torch

    from .batch import ReplicaBatch
    from .rccsd_dense import DeviceERIs
    from .synthetic import WORKLOADS, make_system
    w = WORKLOADS["o20v100x64"]
    system = make_system("o20v100x64", seed=0)
    if args.precision == "split":
        from .cholesky import split_eris
        E = split_eris(system)
    else:
        E = DeviceERIs.from_system(system)
    settings = {"m_keep": w["m"]}
    seeds = [1000 + r for r in range(args.replicas)]
    if args.fused:
        from .replicas import FusedReplicaBatch
        batch = FusedReplicaBatch(E, settings, seeds, precision=args.precision, graph=args.graph)
    else:
        batch = ReplicaBatch(E, settings, seeds, n_streams=args.streams, precision=args.precision,
                             graph=args.graph and not args.batch_graph)
    hist = batch.history
    step = batch.step
    for i in range(args.warmup):
        step()
        if args.batch_graph:  # the first step is eager (it creates the handles), then one graph per batch step
            step = batch.step_graph
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    dt = time.perf_counter() - t
    mean, var = batch.stats()
    burn = min(args.warmup, len(batch.history[0]) - 2)
    tmeans, terrs, taus = batch.trace_stats(burn=max(burn, 0))
    vs_fp64 = None
    if args.vs_fp64 and args.precision != "fp64":
        # the same replicas (same seeds, same number of steps) in FP64: every
        # replica's E_corr at every step against the FP64 batch's
        from .replicas import FusedReplicaBatch
        E64 = DeviceERIs.from_system(system)
        ref = FusedReplicaBatch(E64, settings, seeds, precision="fp64")
        for _ in range(args.warmup + args.steps):
            ref.step()
        d = np.abs(np.array(hist) - np.array(ref.history))
        vs_fp64 = {"max_abs_dE_any_step": float(d.max()), "max_abs_dE_first_step": float(d[:, 0].max()),
                   "steps": int(d.shape[1])}
    return {"mode": "replicas", "workload": "o20v100: nocc=20 nvir=100 naux=600 m=200000 per replica",
            "replicas": args.replicas, "streams": 1 if args.fused else args.streams, "precision": args.precision,
            "form": "fused: one launch per kernel for all replicas" if args.fused else "one solver per replica",
            "graph": ("one graph per batch step" if args.batch_graph or (args.fused and args.graph) else args.graph),
            "iterations_per_s": args.replicas * args.steps / dt, "batch_steps_per_s": args.steps / dt,
            "e_corr_mean": mean, "e_corr_var": var, "iterations_each": args.warmup + args.steps,
            "trace_after_warmup": {"mean_of_means": float(tmeans.mean()), "mcmc_std_median": float(np.median(terrs)),
                                   "tau_median": float(np.median(taus))},
            "vs_fp64": vs_fp64}


def _warm(server, args):
    """One untimed pass of a few requests through the same server: the
    first requests of a process pay one-time set-up (kernel modules loaded
    on first launch, per-thread library handles, allocator growth)."""
    from .batch import request_stream
    warm = request_stream(max(2, min(args.streams, 8)), 1e6, seed=args.seed + 7919,
                          nocc=(args.nocc_min, args.nocc_max))
    server.run(warm, time_scale=0.0)


def run_serve(args):
    import numpy as np

    from .batch import SolveServer, latency_summary, request_stream
    reqs = request_stream(args.requests, args.rate, seed=args.seed, nocc=(args.nocc_min, args.nocc_max))
    server = SolveServer(n_workers=args.streams, precision=args.precision, max_cycle=args.max_cycle, graph=args.graph,
                         device_inputs=not args.host_inputs, rebuild_vvvv=not args.rebuild_once,
                         schedule=args.schedule, max_active=args.max_active, n_builders=args.builders)
    _warm(server, args)
    out = server.run(reqs, time_scale=1.0)
    served = latency_summary(out)
    line = {"mode": "serve", "requests": args.requests, "rate_per_s": args.rate, "schedule": args.schedule,
            "workers": args.streams if args.schedule == "workers" else None,
            "max_active": args.max_active if args.schedule == "iterations" else None,
            "builders": args.builders if args.schedule == "iterations" else None,
            "inputs": "host (numpy)" if args.host_inputs else "device (torch Philox)",
            "vvvv_rebuild": "once per solve" if args.rebuild_once else "every iteration",
            "precision": args.precision, "max_cycle": args.max_cycle, "graph": args.graph, "served": served}
    if args.plain:
        # the same requests, one at a time, FP64, arriving all at once (every
        # --plain-every-th request of the stream: a sample spread evenly over it)
        plain_reqs = request_stream(args.requests, args.rate, seed=args.seed,
                                    nocc=(args.nocc_min, args.nocc_max))[::args.plain_every]
        for r in plain_reqs:
            r.arrival = 0.0
        plain_server = SolveServer(n_workers=1, precision="fp64", max_cycle=args.max_cycle,
                                   device_inputs=not args.host_inputs)
        _warm(plain_server, args)
        plain = plain_server.run(plain_reqs)
        line["plain"] = latency_summary(plain)
        line["plain"]["sample"] = f"every {args.plain_every}th request of the stream ({len(plain_reqs)})"
        by_id = {r.rid: r for r in out}
        diffs = [abs(by_id[b.rid].e_corr - b.e_corr) for b in plain_reqs]
        line["max_abs_dE_vs_plain"] = float(np.max(diffs))
        # one request at a time: the plain arm's rate over the whole stream is
        # one over its mean time per request
        line["speedup_solves_per_s"] = served["solves_per_s"] / line["plain"]["solves_per_s"]
        # the plain arm with its integral builds taken out (one request at a
        # time, so its iterating time is its iterate_s_sum): what the served
        # stream gains on iterating alone, at least (its own span still
        # includes its builds)
        plain_iter = len(plain_reqs) / max(line["plain"]["iterate_s_sum"], 1e-30)
        line["plain"]["solves_per_s_iterating_only"] = plain_iter
        line["speedup_vs_plain_iterating_only"] = served["solves_per_s"] / plain_iter
    return line


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--mode", default="replicas", choices=["replicas", "serve"])
    p.add_argument("--replicas", type=int, default=64)
    p.add_argument("--streams", type=int, default=8)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=1)
    p.add_argument("--precision", default="df64", choices=["fp64", "df64", "split"])
    p.add_argument("--requests", type=int, default=40)
    p.add_argument("--rate", type=float, default=50.0)
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--nocc-min", type=int, default=5)
    p.add_argument("--nocc-max", type=int, default=30)
    p.add_argument("--max-cycle", type=int, default=30)
    p.add_argument("--plain", action="store_true", help="serve: also solve the requests one at a time in plain FP64")
    p.add_argument("--plain-every", type=int, default=1, help="serve: the plain arm solves every k-th request")
    p.add_argument("--schedule", default="iterations", choices=["iterations", "workers"],
                   help="serve: one scheduler thread driving every built request an iteration at a time "
                        "(builder threads make the requests), or --streams worker threads each solving one request "
                        "at a time")
    p.add_argument("--max-active", type=int, default=24, help="serve, iterations: requests built or iterating at once")
    p.add_argument("--builders", type=int, default=2, help="serve, iterations: builder threads")
    p.add_argument("--rebuild-once", action="store_true",
                   help="split precision: rebuild (vv|vv) once per solve instead of every iteration")
    p.add_argument("--host-inputs", action="store_true",
                   help="draw each request's synthetic system with numpy on the host (default: on the GPU)")
    p.add_argument("--graph", action="store_true",
                   help="replay each solver's iteration from a CUDA graph (--fused: the whole batch step, one graph)")
    p.add_argument("--batch-graph", action="store_true",
                   help="replicas: capture every replica's iteration into one CUDA graph per batch step")
    p.add_argument("--vs-fp64", action="store_true",
                   help="replicas: afterwards run the same replicas in FP64 (fused) and report |dE_corr| per step")
    p.add_argument("--fused", action="store_true",
                   help="replicas: one launch per kernel for the whole batch (fp64, df64 or split)")
    args = p.parse_args()
    if args.mode == "serve" and not args.graph:
        # One pool for torch and the library: torch allocates through
        # cudaMallocAsync on the device's default pool, the one the
        # library's own stream-ordered scratch comes from, so memory a
        # finished request frees is there for the next request's library
        # scratch (with torch's caching allocator the two pools grew apart
        # over a long stream of differently sized requests until a library
        # allocation failed).  Set before torch is first imported; not with
        # CUDA graphs, whose multi-threaded captures crashed the host
        # process under this allocator.
        os.environ.setdefault("PYTORCH_CUDA_ALLOC_CONF", "backend:cudaMallocAsync")
    line = run_replicas(args) if args.mode == "replicas" else run_serve(args)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
