#!/usr/bin/env python
"""FRI-CCSD iterations per second on one GB300 (and N independent replicas).

Workload (default): o30v150 -- nocc=30, nvir=150 (o^2 v^2 = 20.25M amplitudes),
Cholesky ERIs with naux=900 and factor entries N(0, 0.03^2/naux), MP2
starting T2, m = 2,000,000 kept amplitudes per FRI compression, two
compressions per iteration.  A step is one FRI-CCSD iteration (update_amps
plus the energy), continuing the trajectory from the MP2 guess.  The
headline runs in FP64 (--precision fp64, the default); the FP32-pair form
(df64) and the split-precision form are measured beside it as secondary
figures, each with its |dE_corr| against the FP64 path for one step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl gb300 (default): the CUDA path.  value = iterations/s with everything
resident in HBM; e2e = the same step through the host entry point
(update_amps_host: numpy amplitudes in, numpy out, copies timed);
served_form = a short served request stream (the metric's solves/s against
the plain FP64 form and p50/p99 latency; --served-requests, 0 to skip).
--impl reference: the reference algorithm on the host cores (the oracle port
of fri-cc's C++ plus numpy for the dense algebra).  Warm-up steps are
sampled iterations: both compressions in full, the dense algebra in full,
and every contraction term on one contiguous block of its outer-index
pairs, scaled by the pair count.  Each timed step is one whole iteration
when the warm-up's estimate puts the timed steps within REF_FULL_BUDGET_S
(--ref-steps auto, the default); otherwise each timed step is a sampled
iteration, the block rotating from step to step (B consecutive steps cover
every pair once), and the line says "extrapolated".
--validate-sample (with --impl reference): one full iteration timed beside
the B block estimates of the same iteration.

Under torchrun (N>1) every rank runs its own replica (different seed) of
the same workload; value = all ranks' iterations / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "FRI-CCSD iter/s and solves/s at |ΔEcorr|≤1e-6 Eh vs plain GPU; p50/p99 latency"
# FP64 / FP32 FMA rates used when the live probe (fricc_gb300.peaks) cannot
# run: the figures that probe gave on a GB300 of this pool (TFLOP/s).
FP64_PEAK_FALLBACK = 1.2557
FP32_PEAK_FALLBACK = 74.2
# DRAM bytes (read + write) per launch of the dominant sparse kernel, from
# one single-pass ncu capture (dram__bytes_read.sum + dram__bytes_write.sum)
# of a whole o30v150 iteration: constants, not measured by this run.
# Keys: (precision, workload) -> {term: bytes per launch}; "mean" is the
# mean over the iteration's launches of that kernel.
SPMM_TRAFFIC_CAPTURED = {
    ("fp64", "o30v150"): {"mean": 3.97e9, "2323": 26.0e9, "XY": 9.64e9, "O3V3": 0.54e9},
    ("df64", "o30v150"): {"2323": 36.1e9, "XY": 13.85e9},
}


def fma_peaks(probe: bool = True) -> dict:
    """FP64 and FP32 FMA rates of this GPU (TFLOP/s), measured now by the
    independent-chain FMA probe (a separate process, before any timed
    work); the recorded pool figures if the probe cannot run."""
    if not probe:
        return {"fp64": FP64_PEAK_FALLBACK, "fp32": FP32_PEAK_FALLBACK, "source": "recorded pool figures"}
    try:
        from fricc_gb300 import peaks
        lines = peaks.run()
        fp64 = max(x["tflops"] for x in lines if x.get("kernel") == "dfma16")
        fp32 = max(x["tflops"] for x in lines if x.get("kernel") == "ffma8")
        return {"fp64": fp64, "fp32": fp32, "source": "measured by this run (FMA probe, fricc_gb300.peaks)"}
    except Exception as ex:  # reported in the line, never fatal
        return {"fp64": FP64_PEAK_FALLBACK, "fp32": FP32_PEAK_FALLBACK,
                "source": f"recorded pool figures (probe failed: {type(ex).__name__})"}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="o30v150")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--served-requests", type=int, default=150,
                   help="requests of the served-stream sample reported as served_form (0: none)")
    p.add_argument("--no-secondary", action="store_true",
                   help="skip the secondary measurements of the other arithmetic forms")
    p.add_argument("--no-peak-probe", action="store_true",
                   help="use the recorded FMA peaks instead of running the FMA probe")
    p.add_argument("--validate-sample", action="store_true",
                   help="with --impl reference: time one iteration in full beside its sampled estimate")
    p.add_argument("--ref-steps", default="auto", choices=["auto", "full", "blocks"],
                   help="with --impl reference: time whole iterations ('full'), block-sampled ones ('blocks'), or "
                        "whole ones when the warm-up's estimate puts the timed steps within the time budget")
    p.add_argument("--graph", action="store_true",
                   help="replay each iteration from one captured CUDA graph (after the first, eager one)")
    p.add_argument("--autotune", action="store_true",
                   help="df64: time the launch configurations of every sparse term and GEMM shape during the "
                        "warm-up and keep the fastest")
    p.add_argument("--precision", default="fp64", choices=["fp64", "df64", "split"],
                   help="arithmetic of the sparse terms: FP64, or FP32 pairs (48-bit products, ~40-bit sums) on the "
                        "FP32 pipe; 'split' also rebuilds (vv|vv) every iteration from the BF16 hi+lo Cholesky "
                        "factor on the tcgen05 tensor cores (split-BF16x3, FP32) and builds (ov|vv), (oo|vv) "
                        "the same way")
    return p.parse_args()


# --------------------------------------------------------------------- helpers
def measured_peaks() -> dict:
    """The machine's measured HBM and BF16 peaks (MEASURED_PEAKS.json beside
    this file), or the earlier GB300 measurement when the file is absent."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "fallback": True}


def dist_setup():
    """(world_size, rank, local_rank) from the torchrun environment."""
    from fricc_gb300.dist import world
    return world()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[3 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def seeded_draws(seed):
    """The reference's stream: srand(seed) then rand()/RAND_MAX per compression."""
    libc = ctypes.CDLL(None)
    libc.srand(ctypes.c_uint(seed))
    libc.rand.restype = ctypes.c_int
    return lambda: float(libc.rand()) / 2147483647.0


# ------------------------------------------------------------------ CPU side
def block_plan(n_outer: int, n_blocks: int, block: int):
    """Block ``block`` of ``n_blocks`` contiguous blocks of a term's outer
    pairs: ((begin, end), size)."""
    begin = (block * n_outer) // n_blocks
    end = ((block + 1) * n_outer) // n_blocks
    return (begin, end), end - begin


class BlockOracle:
    """The oracle port with each contraction term run on one contiguous block
    (block ``block`` of ``n_blocks``) of its outer-index pairs; the term's
    full time is the block's time scaled by the pair count.  A contiguous
    block keeps what the full loop does to the memory system (neighbouring
    pairs share cache lines of W and of the output, and the OpenMP threads
    balance many pairs each); rotating the block from step to step makes the
    estimates of n_blocks consecutive steps add up to whole terms."""

    def __init__(self, n_blocks, block):
        from oracle import fri_oracle
        self.FO = fri_oracle
        self.SparseTensor4d = fri_oracle.SparseTensor4d
        self.n_blocks = n_blocks
        self.block = block % n_blocks
        self.full_below = 0.5  # seconds: a term this cheap runs in full (its fixed costs do not scale)
        self.contract_s = 0.0
        self.sample_wall = 0.0
        self.per_term = {}

    def contract_DTSpT(self, W, T, out, term):
        n_outer = self.FO.outer_size(term, T.dims, W.shape)
        rng, k = block_plan(n_outer, self.n_blocks, self.block)
        t = time.perf_counter()
        if k > 0:
            self.FO.contract_DTSpT(W, T, out, term, outer_range=rng)
        dt = time.perf_counter() - t
        self.sample_wall += dt
        est = dt * n_outer / k if k > 0 else 0.0
        if k < n_outer and est < self.full_below:  # cheap: time the whole term instead
            t = time.perf_counter()
            self.FO.contract_DTSpT(W, T, out, term)
            est = time.perf_counter() - t
            self.sample_wall += est
        self.contract_s += est
        self.per_term[term] = self.per_term.get(term, 0.0) + est


def cpu_sampled_iteration(eris_np, t1, t2, m, n_blocks, block, rn_draw):
    """One reference iteration on the host with every contraction term on
    one block of its outer pairs: seconds (estimated), the wall time actually
    spent, the compression time and the per-term estimates."""
    from oracle import ccsd_oracle as CO
    so = BlockOracle(n_blocks, block)
    settings = {"m_keep": m, "compression": "fri", "sampling_method": "systematic", "verbose": False,
                "compressed_contractions": ["O^2V^4", "O^3V^3", "O^4V^2"]}
    tim = {}
    t0 = time.perf_counter()
    CO.update_amps(settings, t1, t2, eris_np, rn_draw=rn_draw, sparse=so, timings=tim)
    wall = time.perf_counter() - t0
    seconds = wall - so.sample_wall + so.contract_s
    return seconds, wall, tim.get("compress", 0.0), so.per_term


def n_blocks_for(steps: int, cap: int = 10) -> int:
    """Blocks per term for a run of ``steps`` steps: the largest divisor of
    steps up to ``cap`` (so every block is timed equally often), or
    min(steps, cap) when steps has none above 1."""
    best = max(d for d in range(1, min(steps, cap) + 1) if steps % d == 0)
    return best if best > 1 or steps == 1 else min(steps, cap)


def cpu_full_iteration(eris_np, t1, t2, m, rn_draw, amplitudes=False):
    """One reference iteration on the host with every term in full: seconds,
    the per-term times and (``amplitudes``) the new (t1, t2)."""
    from oracle import ccsd_oracle as CO
    settings = {"m_keep": m, "compression": "fri", "sampling_method": "systematic", "verbose": False,
                "compressed_contractions": ["O^2V^4", "O^3V^3", "O^4V^2"]}
    tim = {}
    t0 = time.perf_counter()
    new = CO.update_amps(settings, t1, t2, eris_np, rn_draw=rn_draw, timings=tim)
    secs = time.perf_counter() - t0
    return (secs, tim, new) if amplitudes else (secs, tim)


# The reference arm times whole iterations when the estimate (from its
# warm-up steps) says the timed steps fit in this many seconds; otherwise
# every step runs the block sample.
REF_FULL_BUDGET_S = 1200.0


def _sample_text(workload, cores, n_blocks, wall, steps):
    return (f"each step: one {workload} iteration of the oracle port of fri-cc's C++ (OpenMP, {cores} threads) "
            f"and numpy dense algebra; both compressions and the dense algebra in full; every contraction term on "
            f"one contiguous block of 1/{n_blocks} of its outer-index pairs (block = step mod {n_blocks}, so "
            f"{n_blocks} consecutive steps cover every pair once), its time scaled by the pair count (a term "
            f"estimated under 0.5 s runs in full instead); "
            f"{steps} step(s), {wall:.1f} s of CPU work")


def host_eris_from_device(E):
    from oracle import pyscf_standin as P
    blocks = E.to_numpy_blocks()
    return P._ChemistsERIs(E.fock.cpu().numpy(), E.mo_energy.cpu().numpy(), E.nocc, blocks)


def cpu_baseline_line(eris_np, t1, t2, m, workload, seed, n_blocks=10, blocks=(0, 5)):
    """The reference algorithm on the host cores for the GPU arm's line:
    a bounded sample (two blocks of every term, each with the iteration's
    compressions and dense algebra in full)."""
    from oracle import fri_oracle
    cores = os.cpu_count() or 1
    fri_oracle.set_threads(cores)
    draw = seeded_draws(seed)
    est, walls = [], []
    for b in blocks:
        secs, wall, _, _ = cpu_sampled_iteration(eris_np, t1, t2, m, n_blocks, b, draw)
        est.append(secs)
        walls.append(wall)
    secs = sum(est) / len(est)
    return {"value": 1.0 / secs, "unit": "iter/s", "cores": cores, "kind": "port", "extrapolated": True,
            "sample": _sample_text(workload, cores, n_blocks, sum(walls), len(blocks))
            + f" (blocks {list(blocks)}; {secs:.1f} s/iteration estimated)"}


def served_sample(n_requests: int, timeout_s: float = 420.0) -> dict:
    """The served form on a short stream of the request distribution (split
    precision, iteration-level scheduling) beside the plain FP64 form on
    every 10th of the same requests, one at a time: solves/s, p50/p99 time
    to converged energy and the largest |dE_corr| against the plain form.
    Runs in a child process (its own allocator settings; a failure there
    is reported, never fatal to the headline)."""
    cmd = [sys.executable, "-m", "fricc_gb300.serve_bench", "--mode", "serve", "--requests", str(n_requests),
           "--rate", "50", "--precision", "split", "--schedule", "iterations", "--max-active", "8", "--plain",
           "--plain-every", "10"]
    try:
        r = subprocess.run(cmd, cwd=REPO, capture_output=True, text=True, timeout=timeout_s)
        lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
        if r.returncode != 0 or not lines:
            return {"error": f"serve_bench rc {r.returncode}: {r.stderr[-300:]}"}
        d = json.loads(lines[-1])
    except Exception as ex:
        return {"error": f"{type(ex).__name__}: {str(ex)[:300]}"}
    sv, pl = d["served"], d["plain"]
    return {"unit": "solves/s", "solves_per_s": sv["solves_per_s"], "p50_s": sv["p50_s"], "p99_s": sv["p99_s"],
            "plain_fp64_solves_per_s": pl["solves_per_s"], "speedup_vs_plain_fp64": d["speedup_solves_per_s"],
            "max_abs_dE_vs_plain_fp64": d["max_abs_dE_vs_plain"], "converged": sv["converged"], "requests": sv["n"],
            "workload": (f"{n_requests} requests, Poisson arrivals at 50/s: nocc ~ U{{5..30}}, nvir = ceil(r nocc), "
                         "r ~ U[4,6], naux = 8 (nocc + nvir), kept fraction ~ U[5%, 20%], converged at |dE| < 1e-7 "
                         "Eh; served in split precision at iteration level (one scheduler thread, at most 8 live "
                         "requests); plain arm: every 10th request, one at a time, FP64"),
            "note": ("a short stream: arrivals outpace the server, so p50/p99 include queueing; plain-arm solves/s "
                     "from its 1-in-10 sample")}


WORKLOAD_TEXT = ("{wl}: nocc={o} nvir={v} naux={naux} Cholesky factor entries N(0, {sigma}^2/naux) (a factor "
                 "normalised by naux; entries N(0, {sigma}^2) put every workload outside CCSD's convergence "
                 "regime), m={m} FRI systematic, 2 compressions/iteration, MP2 start")


def workload_text(wl, o, v, w):
    return WORKLOAD_TEXT.format(wl=wl, o=o, v=v, naux=w["naux"], sigma=w["sigma"], m=w["m"])


def secondary_form_line(precision, args, system, E, t1, t2, m, stream):
    """Iterations/s of another arithmetic form on the bench's workload (CUDA
    events over args.steps steps after 2 warm-up steps), its |dE_corr|
    against the FP64 GPU path for one step from the same state and draws,
    and the roofline of its dominant kernel."""
    import torch

    from fricc_gb300 import _lib
    from fricc_gb300.friccsd import FRICCSDGPU
    from fricc_gb300.rng import GlibcRand
    lib = _lib.load()
    if precision == "split":
        from fricc_gb300.cholesky import split_eris
        Es = split_eris(system, device=t2.device)
    else:
        Es = E
    sol = FRICCSDGPU(Es, {"m_keep": m}, rn_draw=GlibcRand(4242), precision=precision)
    a1, a2 = t1, t2
    for _ in range(2):
        a1, a2 = sol.update_amps(a1, a2)
    rn = [0.3141592653589793, 0.2718281828459045]
    sol.update_amps(a1, a2, rn=rn)
    e_form = sol.read_energy()[0]
    ref = FRICCSDGPU(E, {"m_keep": m}, precision="fp64")
    ref.update_amps(a1, a2, rn=rn)
    d_e = abs(ref.read_energy()[0] - e_form)
    del ref
    torch.cuda.synchronize()
    lib.fricc_prof_enable(1)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        a1, a2 = sol.update_amps(a1, a2)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    p_ms, p_n, p_fl = ctypes.c_double(), ctypes.c_longlong(), ctypes.c_double()
    _lib.check(lib.fricc_prof_read(ctypes.byref(p_ms), ctypes.byref(p_n), ctypes.byref(p_fl)))
    t_ms, t_n, t_fl = ctypes.c_double(), ctypes.c_longlong(), ctypes.c_double()
    _lib.check(lib.fricc_prof_read_tc(ctypes.byref(t_ms), ctypes.byref(t_n), ctypes.byref(t_fl)))
    lib.fricc_prof_enable(0)
    sol.read_energy()
    line = {"value": args.steps / (ms / 1000.0), "unit": "iter/s", "ms_per_step": ms / args.steps,
            "delta_e_vs_fp64_per_step": d_e}
    if precision == "split":
        sus = measured_peaks().get("bf16_tflops_sustained")
        ach = t_fl.value / (t_ms.value / 1000.0) / 1e12 if t_ms.value > 0 else None
        line["dtype"] = "split-BF16x3 on tcgen05 (FP32 accumulation); FP64 compression, denominators, energy"
        line["tensor_core"] = {
            "kernel": "k_gemm_tc (all tcgen05 GEMMs of the step)", "achieved": ach, "peak": sus,
            "unit": "TFLOP/s", "frac": (ach / sus) if (ach and sus) else None,
            "flops_counted": "2 M N K' per launch (K' = 3 K): the zero-filled compressed T2 of the sparse "
                             "terms included, so about 90% of the O^2V^4 term's counted flops multiply zeros",
            "share_of_step": t_ms.value / ms if ms > 0 else None, "launches": int(t_n.value)}
    else:
        pk = fma_peaks_cached()["fp32"] / 12.0
        ach = (p_fl.value / (p_ms.value / 1000.0)) / 1e12 if p_ms.value > 0 else None
        line["dtype"] = "f64 storage; sparse terms and dense GEMMs in f32 pairs (48-bit products, ~40-bit sums)"
        line["spmm"] = {"kernel": "k_spmm_df (bucketed sparse-T2 x dense-W, FP32 pairs)", "achieved": ach,
                        "peak": pk, "unit": "TFLOP/s (FP64-equivalent)", "frac": (ach / pk) if ach else None,
                        "peak_source": "FP32 FMA rate / 12 FP32 instructions per FP32-pair multiply-add",
                        "share_of_step": p_ms.value / ms if ms > 0 else None, "launches": int(p_n.value),
                        "traffic_per_launch_captured": SPMM_TRAFFIC_CAPTURED.get((precision, args.workload))}
    del sol
    return line


_PEAKS = None


def fma_peaks_cached(probe: bool = True):
    global _PEAKS
    if _PEAKS is None:
        _PEAKS = fma_peaks(probe)
    return _PEAKS


# ------------------------------------------------------------------ GPU arm
def run_gpu(args):
    world, rank, local = dist_setup()
    if rank == 0:
        fma_peaks_cached(not args.no_peak_probe)  # the FMA probe runs before this process touches the GPU
    import torch
    import torch.distributed as dist

    from fricc_gb300 import _lib
    from fricc_gb300.dist import max_over_ranks, replica_seed
    from fricc_gb300.friccsd import FRICCSDGPU
    from fricc_gb300.rccsd_dense import DeviceERIs
    from fricc_gb300.synthetic import WORKLOADS, make_system

    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = _lib.load()
    w = WORKLOADS[args.workload]
    m = w["m"]
    system = make_system(args.workload, seed=rank)
    E = DeviceERIs.from_system(system, device=dev)
    o, v = system.nocc, system.nvir
    e = E.mo_energy
    eia = e[:o, None] - e[None, o:]
    t2 = (E.ovov.permute(0, 2, 1, 3) / (eia[:, None, :, None] + eia[None, :, None, :])).contiguous()
    t1 = torch.zeros(o, v, dtype=torch.float64, device=dev)
    Es = None
    if args.precision == "split":
        from fricc_gb300.cholesky import split_eris
        Es = split_eris(system, device=dev)
    solver = FRICCSDGPU(Es if Es is not None else E, {"m_keep": m}, rn_draw=seeded_draws(replica_seed(1000, rank)),
                        precision=args.precision, autotune=args.autotune, graph=args.graph)
    stream = torch.cuda.current_stream()

    for _ in range(args.warmup):
        t1, t2 = solver.update_amps(t1, t2)
    torch.cuda.synchronize()

    # |dE_corr| of one step against the plain FP64 GPU path on the same
    # amplitudes and draws (outside the timed region)
    delta_e = None
    if args.precision != "fp64":
        ref_solver = FRICCSDGPU(E, {"m_keep": m}, precision="fp64")
        solver.update_amps(t1, t2, rn=[0.3141592653589793, 0.2718281828459045])
        e_mixed = solver.read_energy()[0]
        ref_solver.update_amps(t1, t2, rn=[0.3141592653589793, 0.2718281828459045])
        delta_e = abs(ref_solver.read_energy()[0] - e_mixed)
        del ref_solver
        torch.cuda.empty_cache()

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    lib.fricc_prof_enable(1)
    launches0 = lib.fricc_launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            t1, t2 = solver.update_amps(t1, t2)
        ev1.record(stream)
        barrier()
    ms = ev0.elapsed_time(ev1)
    launches = lib.fricc_launch_count() - launches0
    p_ms, p_n, p_fl = ctypes.c_double(), ctypes.c_longlong(), ctypes.c_double()
    _lib.check(lib.fricc_prof_read(ctypes.byref(p_ms), ctypes.byref(p_n), ctypes.byref(p_fl)))
    t_ms, t_n, t_fl = ctypes.c_double(), ctypes.c_longlong(), ctypes.c_double()
    _lib.check(lib.fricc_prof_read_tc(ctypes.byref(t_ms), ctypes.byref(t_n), ctypes.byref(t_fl)))
    g_ms, g_n, g_fl = ctypes.c_double(), ctypes.c_longlong(), ctypes.c_double()
    _lib.check(lib.fricc_prof_read_gemm(ctypes.byref(g_ms), ctypes.byref(g_n), ctypes.byref(g_fl)))
    lib.fricc_prof_enable(0)
    energy_last = solver.read_energy()[0]

    ms_max = max_over_ranks(ms, dev)
    value = world * args.steps / (ms_max / 1000.0)

    # end to end through the host entry point: numpy in, numpy out
    e2e = None
    if not args.no_e2e:
        t1h = t1.cpu().numpy().copy()
        t2h = t2.cpu().numpy().copy()
        t1p = torch.from_numpy(t1h).pin_memory().numpy()
        t2p = torch.from_numpy(t2h).pin_memory().numpy()
        solver.update_amps_host(t1p, t2p)  # warm the pinned path
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            t1p, t2p = solver.update_amps_host(t1p, t2p)
        barrier()
        e2e_s = time.perf_counter() - t0
        te = max_over_ranks(e2e_s, dev)
        nb = 8 * (o * v + o * o * v * v)
        e2e = {"value": world * args.steps / te, "unit": "iter/s", "h2d_bytes_per_step": nb,
               "d2h_bytes_per_step": nb}
    del solver
    torch.cuda.empty_cache()

    # the other arithmetic forms on the same workload, as secondary figures
    # (narrower arithmetic than FP64, so never the headline), each with its
    # |dE| against the FP64 path for one step from the same state and draws
    secondary = {}
    if world == 1 and not args.no_secondary:
        for form in ("df64", "split"):
            if form == args.precision:
                continue
            try:
                secondary[form + "_form"] = secondary_form_line(form, args, system, E, t1, t2, m, stream)
            except Exception as ex:  # reported, never fatal to the headline
                secondary[form + "_form"] = {"error": f"{type(ex).__name__}: {str(ex)[:300]}"}
            torch.cuda.empty_cache()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        eris_np = host_eris_from_device(E)
        t1h, t2h = system.mp2_amplitudes()
        cpu = cpu_baseline_line(eris_np, t1h, t2h, m, args.workload, 7)

    # the served request stream (the metric's solves/s and p50/p99), a
    # short sample in a child process
    served = None
    if rank == 0 and world == 1 and args.served_requests > 0:
        torch.cuda.empty_cache()
        served = served_sample(args.served_requests)

    pk = fma_peaks_cached() if rank == 0 else {"fp64": FP64_PEAK_FALLBACK, "fp32": FP32_PEAK_FALLBACK,
                                                "source": "recorded pool figures"}
    achieved = (p_fl.value / (p_ms.value / 1000.0)) / 1e12 if p_ms.value > 0 else None
    if args.precision == "fp64":
        kname, bound, peak = "k_spmm (bucketed sparse-T2 x dense-W, FP64)", "fp64-pipe", pk["fp64"]
        psrc = f"FP64 FMA rate of this GPU, {pk['source']}; MEASURED_PEAKS.json has no FP64 figure"
    elif args.precision == "split":
        kname, bound, peak = "k_spmm_f32 (bucketed sparse-T2 x dense-W, FP32; terms too small for the tensor cores)", \
            "fp32-pipe", pk["fp32"]
        psrc = f"FP32 FMA rate of this GPU, {pk['source']}: one packed FMA per two outputs"
    else:
        kname, bound, peak = "k_spmm_df (bucketed sparse-T2 x dense-W, FP32 pairs)", "fp32-pipe", pk["fp32"] / 12
        psrc = (f"FP32 FMA rate of this GPU ({pk['source']}) / 12 FP32 instructions per FP32-pair multiply-add, "
                "counted as 2 FP64-equivalent flops")
    traffic = SPMM_TRAFFIC_CAPTURED.get((args.precision, args.workload))
    roof = {"kernel": kname, "bound": bound,
            "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": (achieved / peak) if achieved else None,
            "traffic": traffic.get("mean") if traffic else None,
            "traffic_per_launch_captured": traffic,
            "traffic_note": ("DRAM bytes per launch (mean over the iteration's launches of the kernel) from one "
                             "single-pass ncu capture of an iteration of this workload with this build, not measured "
                             "by this run; the 2323 launch re-reads its W' (algorithmic 4.37 GB) ~6x without "
                             "costing time: the kernel is bound by the FP64 pipe, not DRAM"),
            "flops_counted": "2 m Q per launch (m nonzeros, Q outputs per nonzero): algorithmic, no padding",
            "launches": int(p_n.value), "kernel_ms": p_ms.value,
            "kernel_share_of_step": p_ms.value / ms if ms > 0 else None,
            "peak_source": psrc}
    gemm = None
    if g_n.value:
        g_ach = (g_fl.value / (g_ms.value / 1000.0)) / 1e12 if g_ms.value > 0 else None
        gemm = {"kernel": "k_gemm_f64 (dense O^2V^3 / O^3V^2 contractions, FP64 DFMA)", "bound": "fp64-pipe",
                "achieved": g_ach, "peak": pk["fp64"], "unit": "TFLOP/s",
                "frac": (g_ach / pk["fp64"]) if g_ach else None, "launches": int(g_n.value),
                "kernel_ms": g_ms.value, "kernel_share_of_step": g_ms.value / ms if ms > 0 else None}
    if args.precision == "split":
        # the dominant kernel of the split form: the tensor-core GEMMs
        sus = measured_peaks().get("bf16_tflops_sustained")
        tc_ach = (t_fl.value / (t_ms.value / 1000.0)) / 1e12 if t_ms.value > 0 else None
        sparse_roof = roof
        roof = {"kernel": "k_gemm_tc (tcgen05 split-BF16x3 GEMMs: the sparse terms on the zero-filled compressed "
                          "T2, the dense algebra, the (vv|vv) rebuild)",
                "bound": "tensor", "achieved": tc_ach, "peak": sus, "unit": "TFLOP/s",
                "frac": (tc_ach / sus) if (tc_ach and sus) else None, "traffic": None,
                "launches": int(t_n.value), "kernel_ms": t_ms.value,
                "kernel_share_of_step": t_ms.value / ms if ms > 0 else None,
                "flops_counted": "2 M N K' per launch (K' = 3 K, the three BF16 products; zero padding and the "
                                 "zeros of the compressed T2 included: about 90% of the O^2V^4 term's counted "
                                 "flops multiply zeros)",
                "peak_source": "bf16_tflops_sustained of MEASURED_PEAKS.json (kernels timed inside the step)",
                "sparse_kernel": sparse_roof if sparse_roof.get("launches") else None}
    dtypes = {"fp64": "f64",
              "df64": "f64 storage; sparse terms and dense GEMMs in f32 pairs (48-bit products, ~40-bit sums)",
              "split": ("f64 (compression, denominators, energy); (vv|vv), (ov|vv), (oo|vv) and the large "
                        "contractions split-BF16x3 on tcgen05 with FP32 accumulation")}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "iter/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": dtypes[args.precision], "data": "synthetic",
            "config": {"workload": workload_text(args.workload, o, v, w),
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "l2": (f"working set > L2: the (ac|bd) block ({8 * v ** 4 / 1e9:.2f} GB FP64) is streamed "
                              "by the O^2V^4 term every step" if args.precision != "split" else
                              "working set > L2: (ac|bd) rebuilt every step as a split-BF16x3 operand "
                              f"({12 * v ** 4 / 1e9:.2f} GB) and streamed by the O^2V^4 GEMM"),
                       "precision": args.precision, "autotune": bool(args.autotune),
                       "cuda_graph": bool(args.graph)},
            "e2e": e2e, "gpu_launches": int(launches), "roofline": roof, "cpu_baseline": cpu,
            "clocks": clk.summary(), "energy_last": energy_last,
            "delta_e_vs_fp64_per_step": delta_e,
        }
        if gemm is not None:
            line["dense_gemm"] = gemm
        line.update(secondary)
        if served is not None:
            line["served_form"] = served
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


# ------------------------------------------------------------------ reference arm
def run_reference(args):
    world, rank, local = dist_setup()
    if rank != 0:
        return
    from oracle import fri_oracle, pyscf_standin as P
    from fricc_gb300.synthetic import WORKLOADS, make_system

    fri_oracle.build()
    cores = os.cpu_count() or 1
    fri_oracle.set_threads(cores)
    w = WORKLOADS[args.workload]
    system = make_system(args.workload, seed=0)
    eris_np = None
    try:  # the GPU builds the 4 GB integral set in a second; the host in minutes
        import torch
        if torch.cuda.is_available():
            from fricc_gb300.rccsd_dense import DeviceERIs
            eris_np = host_eris_from_device(DeviceERIs.from_system(system))
            torch.cuda.empty_cache()
    except Exception:
        eris_np = None
    if eris_np is None:
        eris_np = P.make_eris(system)
    t1, t2 = system.mp2_amplitudes()
    m = w["m"]
    n_blocks = n_blocks_for(args.steps)
    if args.validate_sample:
        # the same iteration (same amplitudes and draws) in full, and as the
        # n_blocks block estimates a run of that many steps adds up
        full, per_full = cpu_full_iteration(eris_np, t1, t2, m, seeded_draws(1000))
        blocks = []
        per_blocks = {}
        for b in range(n_blocks):
            est, wall, _, per = cpu_sampled_iteration(eris_np, t1, t2, m, n_blocks, b, seeded_draws(1000))
            blocks.append({"block": b, "estimate_s": est, "wall_s": wall})
            for k, v in per.items():
                per_blocks[k] = per_blocks.get(k, 0.0) + v / n_blocks
        mean_est = sum(x["estimate_s"] for x in blocks) / n_blocks
        print(json.dumps({"validate_sample": args.workload, "cores": cores, "n_blocks": n_blocks,
                          "full_s": full, "mean_block_estimate_s": mean_est,
                          "ratio_estimate_over_full": mean_est / full, "blocks": blocks,
                          "terms_mean_estimate_s": per_blocks,
                          "terms_full_s": {k: v for k, v in per_full.items() if k != "compress"},
                          "compress_s": per_full.get("compress")}))
        return
    draw = seeded_draws(1000)
    # warm-up: block-sampled iterations (every code path of the iteration
    # runs once per step); their estimates decide whether the timed steps
    # can run whole iterations within the budget
    n_warm_blocks = 10
    warm_est = []
    for step in range(args.warmup):
        secs, _, _, _ = cpu_sampled_iteration(eris_np, t1, t2, m, n_warm_blocks, step, draw)
        warm_est.append(secs)
    est = min(warm_est) if warm_est else float("inf")
    full = args.ref_steps == "full" or (args.ref_steps == "auto" and est * args.steps <= REF_FULL_BUDGET_S)
    per = []
    walls = []
    for step in range(args.steps):
        if full:  # whole iterations, continuing the trajectory from the MP2 start
            secs, _, (t1, t2) = cpu_full_iteration(eris_np, t1, t2, m, draw, amplitudes=True)
            wall = secs
        else:
            secs, wall, _, _ = cpu_sampled_iteration(eris_np, t1, t2, m, n_blocks, step, draw)
        per.append(secs)
        walls.append(wall)
    total = sum(per)
    value = args.steps / total
    if full:
        sample = (f"each step: one whole {args.workload} iteration of the oracle port of fri-cc's C++ (OpenMP, "
                  f"{cores} threads) and numpy dense algebra, continuing the trajectory from the MP2 start; "
                  f"{args.steps} step(s), {total:.1f} s of CPU work timed (warm-up: {args.warmup} block-sampled "
                  f"iteration(s), estimate {est:.1f} s/iteration)")
    else:
        sample = _sample_text(args.workload, cores, n_blocks, sum(walls), args.steps)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "iter/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total / args.steps,
        "timed_wall_ms_per_step": 1000.0 * sum(walls) / args.steps, "extrapolated": not full,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_text(args.workload, system.nocc, system.nvir, w),
                   "parallelism": "host cores", "precision": "fp64"},
        "cpu_baseline": {"value": value, "unit": "iter/s", "cores": cores, "kind": "port", "extrapolated": not full,
                         "sample": sample},
        "e2e": {"value": value, "unit": "iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
