"""Launch schedules of the float-pair sparse kernel on a workload's own terms
(python -m fricc_gb300.spmm_schedules).

Builds the workload's integrals and MP2 amplitudes, compresses T2 once
(m of the workload, systematic FRI), and times ``fricc_spmm_f2`` on the
2323 term ((ac|bd), Q = v^2), the X/Y t1 parts of Wvvvv (Q = 2ov) and one
O^3V^3 pass (0313+0113, Q = ov) under each launch configuration given (the
library's tune knobs: 0 = output pairs per thread, 5 = the persistent
q-tile-major launch's CTAs per SM): CUDA events around each launch, the
best of ``--reps`` after one warm-up, and whether the output equals the
default configuration's bit for bit.  One JSON line per (term,
configuration).

    python -m fricc_gb300.spmm_schedules [--workload o30v150] [--terms 2323,XY,0313]
        [--configs '[{}, {"5": 4, "0": 2}]'] [--reps 4]
"""
from __future__ import annotations

import argparse
import ctypes
import json

DEFAULT_CONFIGS = [{}] + [{0: p} for p in (1, 4)] + [{5: k, 0: p} for k in (2, 3, 4, 6, 8) for p in (1, 2)]


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--workload", default="o30v150")
    p.add_argument("--terms", default="2323,XY,0313")
    p.add_argument("--configs", default=None, help="JSON list of {knob: value} (default: the full sweep)")
    p.add_argument("--reps", type=int, default=4)
    args = p.parse_args()

    import torch

    from . import _lib as L
    from .autotune import knobs
    from .batch import mp2_device
    from .friccsd import _Handle
    from .rccsd_dense import DeviceERIs
    from .synthetic import WORKLOADS, make_system

    cfgs = DEFAULT_CONFIGS if args.configs is None else \
        [{int(k): v for k, v in c.items()} for c in json.loads(args.configs)]
    E = DeviceERIs.from_system(make_system(args.workload, seed=0))
    E.prepare_splits()
    t1, t2 = mp2_device(E)
    o, v = t1.shape
    st = L.cur_stream()
    h = _Handle()
    h.compress(t2, WORKLOADS[args.workload]["m"], "fri", 0.5, st)
    lib = L.load()
    ov = o * v
    terms = {"2323": (0, 1, 2, 3, "vvvvT", v * v, o * o * v * v),
             "XY": (0, 1, 2, 3, "ovvv_XY", 2 * ov, o * o * 2 * ov),
             "0313": (2, 0, 1, 3, "ovov_0313_0113", ov, o * o * v * v)}
    Op = torch.zeros(o * o * v * v * 2, dtype=torch.float64, device="cuda")
    for name in args.terms.split(","):
        pa, pb, ka, kb, const, QS, nout = terms[name]
        W2 = E.split(const)
        ref = None
        for cfg in cfgs:
            def launch():
                L.check(lib.fricc_spmm_f2(h.h, pa, pb, ka, kb, 1.0, ctypes.c_void_p(W2.data_ptr()), int(QS),
                                          ctypes.c_void_p(Op.data_ptr()), st))
            with knobs(cfg):
                Op[:nout].zero_()
                launch()
                ts = []
                for _ in range(max(1, args.reps)):
                    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    Op[:nout].zero_()
                    a.record()
                    launch()
                    b.record()
                    b.synchronize()
                    ts.append(a.elapsed_time(b))
                out = Op[:nout].clone()
            if ref is None:
                ref = out
            same = bool(torch.equal(out.view(torch.int64), ref.view(torch.int64)))
            print(json.dumps({"term": name, "config": {str(k): x for k, x in cfg.items()}, "ms": min(ts),
                              "bit_identical_to_first": same}), flush=True)


if __name__ == "__main__":
    main()
