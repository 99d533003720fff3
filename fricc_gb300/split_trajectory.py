"""|dE_corr| of the split-precision form along a whole FRI-CCSD trajectory
(python -m fricc_gb300.split_trajectory --workload o40v200 --iters 40).

Both runs start from the MP2 amplitudes of the same synthetic system and take
the same draws (one GlibcRand stream per run, same seed), so they sample the
same way as long as the amplitudes agree; the split-precision run
(integrals rebuilt from the BF16 hi+lo Cholesky factor on the tensor cores)
is compared iteration by iteration with the plain FP64 GPU path.  One JSON
line: the energies' largest and final |dE|, both runs' final E_corr, and the
split run's iterations/s.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch

from .batch import mp2_device
from .cholesky import split_eris
from .friccsd import FRICCSDGPU
from .rccsd_dense import DeviceERIs
from .rng import GlibcRand
from .synthetic import WORKLOADS, make_system


def trajectory(solver, E, iters):
    t1, t2 = mp2_device(E)
    out = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(iters):
        t1, t2 = solver.update_amps(t1, t2)
        out.append(solver.read_energy()[0])
    torch.cuda.synchronize()
    return np.array(out), time.perf_counter() - t0


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--workload", default="o40v200")
    p.add_argument("--iters", type=int, default=None)
    p.add_argument("--seed", type=int, default=2024)
    p.add_argument("--reference", default="fp64", choices=["fp64", "df64"])
    args = p.parse_args()
    w = WORKLOADS[args.workload]
    iters = args.iters or w["iters"]
    system = make_system(args.workload, seed=0)
    settings = {"m_keep": w["m"]}
    Es = split_eris(system)
    e_split, t_split = trajectory(FRICCSDGPU(Es, settings, rn_draw=GlibcRand(args.seed), precision="split"), Es, iters)
    del Es
    torch.cuda.empty_cache()
    E = DeviceERIs.from_system(system)
    e_ref, t_ref = trajectory(FRICCSDGPU(E, settings, rn_draw=GlibcRand(args.seed), precision=args.reference), E, iters)
    d = np.abs(e_split - e_ref)
    print(json.dumps({
        "workload": args.workload, "iterations": iters, "m": w["m"], "reference": args.reference,
        "max_abs_dE": float(d.max()), "final_abs_dE": float(d[-1]),
        "e_corr_final_split": float(e_split[-1]), "e_corr_final_reference": float(e_ref[-1]),
        "split_iter_per_s": iters / t_split, "reference_iter_per_s": iters / t_ref,
        "abs_dE_by_iteration": [float(x) for x in d],
    }))


if __name__ == "__main__":
    main()
