#!/usr/bin/env python
"""FRI-CCSD iterations per second on one GB300 (and N independent replicas).

Workload (default): o30v150 -- nocc=30, nvir=150 (o^2 v^2 = 20.25M amplitudes),
Cholesky ERIs with naux=900 and N(0, 0.03^2) entries, MP2 starting T2,
m = 2,000,000 kept amplitudes per FRI compression, two compressions per
iteration, FP64 throughout.  A step is one FRI-CCSD iteration (update_amps
plus the energy), continuing the trajectory from the MP2 guess.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl gb300 (default): the CUDA path.  value = iterations/s with everything
resident in HBM; e2e = the same step through the host entry point
(update_amps_host: numpy amplitudes in, numpy out, copies timed).
--impl reference: the reference algorithm on the host cores (the oracle port
of fri-cc's C++ plus numpy for the dense algebra), each step one sampled
iteration: both compressions in full, the dense algebra in full, and every
contraction term on a bounded sample of its outer-index pairs, scaled by the
pair count.

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
# FP64 and FP32 FMA throughput of this GB300 pool, measured with the
# independent-chain FMA probe of fricc_gb300/peaks.cu (python -m
# fricc_gb300.peaks; profiles/fp64_peak_gb300.md): the contraction kernels are
# FP64- or FP32-pipe bound and MEASURED_PEAKS.json has no figure for either.
FP64_PEAK_TFLOPS = 1.2557
FP32_PEAK_TFLOPS = 74.2
# DRAM bytes (read + write) per k_spmm_df launch, df64, from one ncu capture
# of an o30v150 iteration's ten launches (profiles/k_spmm_df_traffic_o30v150.md):
# 54.30 GB in total, of which 36.1 GB in the 2323 launch and 13.9 GB in X/Y.
SPMM_TRAFFIC = {"o30v150": 5.43e9}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="o30v150")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-split-form", action="store_true",
                   help="skip the secondary measurement of the split-precision form")
    p.add_argument("--graph", action="store_true",
                   help="replay each iteration from one captured CUDA graph (after the first, eager one)")
    p.add_argument("--autotune", action="store_true",
                   help="df64: time the launch configurations of every sparse term and GEMM shape during the "
                        "warm-up and keep the fastest")
    p.add_argument("--precision", default="df64", choices=["fp64", "df64", "split"],
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
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


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
class SampledOracle:
    """The oracle port with each contraction term run on a bounded sample of
    its outer-index pairs; the term's full time is the sample's time scaled
    by the pair count (the reference's cost per pair is the same m-entry scan
    plus that pair's nonzeros)."""

    def __init__(self, pairs_per_term):
        from oracle import fri_oracle
        self.FO = fri_oracle
        self.SparseTensor4d = fri_oracle.SparseTensor4d
        self.pairs = pairs_per_term
        self.full_below = 1.0  # seconds: a term this cheap runs in full
        self.contract_s = 0.0
        self.sample_wall = 0.0

    def contract_DTSpT(self, W, T, out, term):
        n_outer = self.FO.outer_size(term, T.dims, W.shape)
        k = min(n_outer, self.pairs)
        t = time.perf_counter()
        self.FO.contract_DTSpT(W, T, out, term, outer_range=(0, k))
        dt = time.perf_counter() - t
        self.sample_wall += dt
        est = dt * n_outer / k
        if k < n_outer and est < self.full_below:  # cheap enough: time the whole term instead
            t = time.perf_counter()
            self.FO.contract_DTSpT(W, T, out, term)
            dt = time.perf_counter() - t
            self.sample_wall += dt
            est = dt
        self.contract_s += est


def cpu_sampled_iteration(eris_np, t1, t2, m, pairs, rn_draw):
    """One reference iteration on the host: seconds (extrapolated) and a description."""
    from oracle import ccsd_oracle as CO
    so = SampledOracle(pairs)
    settings = {"m_keep": m, "compression": "fri", "sampling_method": "systematic", "verbose": False,
                "compressed_contractions": ["O^2V^4", "O^3V^3", "O^4V^2"]}
    tim = {}
    t0 = time.perf_counter()
    CO.update_amps(settings, t1, t2, eris_np, rn_draw=rn_draw, sparse=so, timings=tim)
    wall = time.perf_counter() - t0
    seconds = wall - so.sample_wall + so.contract_s
    return seconds, wall, tim.get("compress", 0.0)


def _sample_text(workload, cores, pairs, wall):
    return (f"each step: one {workload} iteration of the oracle port of fri-cc's C++ (OpenMP, {cores} threads) "
            f"and numpy dense algebra; both compressions and the dense algebra in full; each contraction term in "
            f"full when that takes under 1 s, else on its first {pairs} outer-index pairs scaled by the pair "
            f"count; {wall:.1f} s of CPU work")


def host_eris_from_device(E):
    from oracle import pyscf_standin as P
    blocks = E.to_numpy_blocks()
    return P._ChemistsERIs(E.fock.cpu().numpy(), E.mo_energy.cpu().numpy(), E.nocc, blocks)


def cpu_baseline_line(eris_np, t1, t2, m, workload, seed):
    from oracle import fri_oracle
    cores = os.cpu_count() or 1
    fri_oracle.set_threads(cores)
    pairs = 4 * cores
    secs, wall, comp = cpu_sampled_iteration(eris_np, t1, t2, m, pairs, seeded_draws(seed))
    return {"value": 1.0 / secs, "unit": "iter/s", "cores": cores, "kind": "port",
            "sample": _sample_text(workload, cores, pairs, wall) + f" ({secs:.1f} s/iteration extrapolated)"}


def split_form_line(args, system, E, t1, t2, m, stream):
    """Iterations/s of the split-precision form on the bench's workload
    (CUDA events over args.steps steps after 2 warm-up steps), its |dE|
    against the FP64 GPU path, and its tensor-core roofline."""
    import torch

    from fricc_gb300 import _lib
    from fricc_gb300.cholesky import split_eris
    from fricc_gb300.friccsd import FRICCSDGPU
    from fricc_gb300.rng import GlibcRand
    lib = _lib.load()
    Es = split_eris(system, device=t2.device)
    sol = FRICCSDGPU(Es, {"m_keep": m}, rn_draw=GlibcRand(4242), precision="split")
    a1, a2 = t1, t2
    for _ in range(2):
        a1, a2 = sol.update_amps(a1, a2)
    rn = [0.3141592653589793, 0.2718281828459045]
    sol.update_amps(a1, a2, rn=rn)
    e_split = sol.read_energy()[0]
    ref = FRICCSDGPU(E, {"m_keep": m}, precision="fp64")
    ref.update_amps(a1, a2, rn=rn)
    d_e = abs(ref.read_energy()[0] - e_split)
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
    t_ms, t_n, t_fl = ctypes.c_double(), ctypes.c_longlong(), ctypes.c_double()
    _lib.check(lib.fricc_prof_read_tc(ctypes.byref(t_ms), ctypes.byref(t_n), ctypes.byref(t_fl)))
    lib.fricc_prof_enable(0)
    sol.read_energy()
    sus = measured_peaks().get("bf16_tflops_sustained")
    ach = t_fl.value / (t_ms.value / 1000.0) / 1e12 if t_ms.value > 0 else None
    return {"value": args.steps / (ms / 1000.0), "unit": "iter/s", "ms_per_step": ms / args.steps,
            "delta_e_vs_fp64_per_step": d_e,
            "dtype": "split-BF16x3 on tcgen05 (FP32 accumulation); FP64 compression, denominators, energy",
            "tensor_core": {"kernel": "k_gemm_tc (all tcgen05 GEMMs of the step)", "achieved": ach, "peak": sus,
                            "unit": "TFLOP/s", "frac": (ach / sus) if (ach and sus) else None,
                            "share_of_step": t_ms.value / ms if ms > 0 else None, "launches": int(t_n.value)}}


# ------------------------------------------------------------------ GPU arm
def run_gpu(args):
    import torch
    import torch.distributed as dist

    from fricc_gb300 import _lib
    from fricc_gb300.friccsd import FRICCSDGPU
    from fricc_gb300.rccsd_dense import DeviceERIs
    from fricc_gb300.synthetic import WORKLOADS, make_system

    world, rank, local = dist_setup()
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
    solver = FRICCSDGPU(Es if Es is not None else E, {"m_keep": m}, rn_draw=seeded_draws(1000 + rank),
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

    # the tensor-core rebuild of (vv|vv) alone (split precision): CUDA events
    # around 3 rebuilds into the solver's own buffer, outside the timed region
    tc_roof = None
    if Es is not None:
        R = Es.vvvv_rebuild
        dense = solver._vvvv_bt is not None  # the rebuild the solver uses
        rebuild = (lambda: R.rebuild_split_b(solver._vvvv_bt)) if dense else (lambda: R.rebuild(solver._vvvv_buf))
        ra, rb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        rebuild()
        ra.record(stream)
        for _ in range(3):
            rebuild()
        rb.record(stream)
        torch.cuda.synchronize()
        R.check()
        r_ms = ra.elapsed_time(rb) / 3
        pk = measured_peaks().get("bf16_tflops")
        ach = R.flops() / (r_ms / 1000.0) / 1e12
        tc_roof = {"kernel": ("k_gemm_tc<EpiVvvvSplitB>" if dense else "k_gemm_tc<EpiVvvv>")
                   + " ((vv|vv) rebuild, tcgen05 BF16, split-BF16x3, FP32 accumulation)",
                   "bound": "tensor", "achieved": ach, "peak": pk, "unit": "TFLOP/s",
                   "frac": ach / pk if pk else None, "ms": r_ms,
                   "flops": R.flops(), "peak_source": "bf16_tflops (burst) of MEASURED_PEAKS.json"}

    lib.fricc_prof_enable(1)
    launches0 = lib.fricc_launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    energies = []
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
    lib.fricc_prof_enable(0)
    energies.append(solver.read_energy()[0])

    t_max = torch.tensor([ms], dtype=torch.float64, device=dev)
    if world > 1:
        dist.all_reduce(t_max, op=dist.ReduceOp.MAX)
    ms_max = float(t_max.item())
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
        te = torch.tensor([e2e_s], dtype=torch.float64, device=dev)
        if world > 1:
            dist.all_reduce(te, op=dist.ReduceOp.MAX)
        nb = 8 * (o * v + o * o * v * v)
        e2e = {"value": world * args.steps / float(te.item()), "unit": "iter/s", "h2d_bytes_per_step": nb,
               "d2h_bytes_per_step": nb}

    # the split-precision form on the same workload, as a secondary figure:
    # integrals rebuilt from the BF16 hi+lo factor and every large
    # contraction on the tcgen05 tensor cores (a different arithmetic, so not
    # the headline); |dE| against the FP64 path for one step from the same
    # state and draws
    split_form = None
    if args.precision == "df64" and world == 1 and not args.no_split_form:
        try:
            split_form = split_form_line(args, system, E, t1, t2, m, stream)
        except Exception as ex:  # reported, never fatal to the headline
            split_form = {"error": f"{type(ex).__name__}: {str(ex)[:300]}"}
        torch.cuda.empty_cache()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        eris_np = host_eris_from_device(E)
        t1h, t2h = system.mp2_amplitudes()
        cpu = cpu_baseline_line(eris_np, t1h, t2h, m, args.workload, 7)

    achieved = (p_fl.value / (p_ms.value / 1000.0)) / 1e12 if p_ms.value > 0 else None
    if args.precision == "fp64":
        kname, bound, peak = "k_spmm (bucketed sparse-T2 x dense-W, FP64)", "fp64", FP64_PEAK_TFLOPS
        psrc = "measured FP64 FMA rate of this GB300 pool (DFMA probe); FP64 is not in MEASURED_PEAKS.json"
    elif args.precision == "split":
        kname, bound, peak = "k_spmm_f32 (bucketed sparse-T2 x dense-W, FP32; terms too small for the tensor cores)", \
            "fp32-pipe", FP32_PEAK_TFLOPS
        psrc = ("FP32 FMA rate of this GB300 pool (74.2 TF/s, FFMA probe): one packed FMA per two outputs, "
                "2 flops per multiply-add")
    else:
        kname, bound, peak = "k_spmm_df (bucketed sparse-T2 x dense-W, FP32 pairs)", "fp32-pipe", FP32_PEAK_TFLOPS / 12
        psrc = ("FP32 FMA rate of this GB300 pool (74.2 TF/s = 37.1 T instructions/s, FFMA probe) / 12 FP32 "
                "instructions per FP32-pair multiply-add, counted as 2 FP64-equivalent flops")
    roof = {"kernel": kname, "bound": bound,
            "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": (achieved / peak) if achieved else None,
            "traffic": SPMM_TRAFFIC.get(args.workload) if args.precision == "df64" else None,
            "launches": int(p_n.value), "kernel_ms": p_ms.value,
            "kernel_share_of_step": p_ms.value / ms if ms > 0 else None,
            "peak_source": psrc}
    if args.precision == "split":
        # the dominant kernel of the split form: the tensor-core GEMMs
        # (dense sparse terms, dense algebra, (vv|vv) rebuild), timed live
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
                                 "zeros of the compressed T2 included)",
                "peak_source": "bf16_tflops_sustained of MEASURED_PEAKS.json (kernels timed inside the step)",
                "sparse_kernel": sparse_roof if sparse_roof.get("launches") else None}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "iter/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "f64 (sparse terms in f32 pairs: 48-bit products, ~40-bit sums)",
            "data": "synthetic",
            "config": {"workload": f"{args.workload}: nocc={o} nvir={v} naux={w['naux']} sigma={w['sigma']} "
                                   f"m={m} FRI systematic, 2 compressions/iteration, FP64",
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "l2": f"working set > L2 ((ac|bd) {8 * v ** 4 / 1e9:.2f} GB and its float-pair copy "
                             "streamed by the O^2V^4 term every step)",
                       "precision": args.precision, "autotune": bool(args.autotune),
                       "cuda_graph": bool(args.graph)},
            "e2e": e2e, "gpu_launches": int(launches), "roofline": roof, "cpu_baseline": cpu,
            "clocks": clk.summary(), "energy_last": energies[-1],
            "delta_e_vs_fp64_per_step": delta_e,
        }
        if split_form is not None:
            line["split_form"] = split_form
        if tc_roof is not None:
            line["tensor_core_rebuild"] = tc_roof
            line["dtype"] = ("f64 (compression, denominators, energy); (vv|vv), (ov|vv), (oo|vv) split-BF16x3 on "
                             "tcgen05 with FP32 accumulation; sparse terms in f32 pairs")
            line["config"]["l2"] = (f"working set > L2 ((ac|bd) rebuilt in FP32, {4 * v ** 4 / 1e9:.2f} GB, "
                                    "streamed by the O^2V^4 term every step)")
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
    pairs = 4 * cores
    draw = seeded_draws(1000)
    # warm-up: one small compression (the CPU path has nothing to warm)
    for _ in range(args.warmup):
        fri_oracle.fri_compression(t2.ravel()[:100000], 1000, rn=0.5)
    per = []
    walls = []
    for _ in range(args.steps):
        secs, wall, _ = cpu_sampled_iteration(eris_np, t1, t2, m, pairs, draw)
        per.append(secs)
        walls.append(wall)
    total = sum(per)
    value = args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "iter/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.workload}: nocc={system.nocc} nvir={system.nvir} naux={w['naux']} "
                               f"sigma={w['sigma']} m={m} FRI systematic, 2 compressions/iteration, FP64",
                   "parallelism": "host cores"},
        "cpu_baseline": {"value": value, "unit": "iter/s", "cores": cores, "kind": "port",
                         "sample": _sample_text(args.workload, cores, pairs, sum(walls))},
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
