"""Per-shape launch-configuration autotuning.

The library exposes thread-local overrides of its launch configurations
(``fricc_tune_set``): the float-pair sparse kernel's output pairs per thread,
the FP32-pair GEMM's tile shape and split-K target, and the width of the
compression's first select digit (how many candidates its exact top-m sort
takes).  ``Autotuner`` times
every candidate configuration of an operation the first time it meets that
operation's shape -- on scratch copies of the outputs, so the real result is
computed once, after the choice -- and replays the fastest configuration for
that shape from then on.  Timing uses CUDA events on the current stream,
best of ``reps`` after one warm-up launch.
"""
from __future__ import annotations

import contextlib
import itertools
import time

import torch

from . import _lib as L

SPMM_PPT, GEMM_TILE, GEMM_COVER, SELECT_BITS, SPMM_PERSIST = 0, 1, 2, 4, 5

# candidate configurations: {knob: value}; {} is the library's own choice.
# The sparse kernel's gather tiles: pairs per thread (the q tile of a CTA is
# 256 x that many outputs), each as one CTA per (bucket, q tile) item or as
# a persistent q-tile-major launch of 8 CTAs per SM
SPMM_CANDIDATES = [{SPMM_PPT: p} for p in (1, 2, 4)] + [{SPMM_PPT: p, SPMM_PERSIST: 8} for p in (1, 2)]
GEMM_CANDIDATES = [{}] + [{GEMM_TILE: t, GEMM_COVER: c} for t, c in itertools.product(range(5), (2, 4, 8))]
# the compression's top-m selection schedule: the first select digit's width
# (candidates left for the exact sort), 12 bits by default
COMPRESS_CANDIDATES = [{SELECT_BITS: b} for b in (10, 11, 12, 13)]


@contextlib.contextmanager
def knobs(cfg: dict):
    """Set the overrides of ``cfg`` for the launches inside the block."""
    lib = L.load()
    try:
        for k, v in cfg.items():
            L.check(lib.fricc_tune_set(int(k), int(v)))
        yield
    finally:
        for k in cfg:
            lib.fricc_tune_set(int(k), -1)


def _cuda_timer(fn):
    s = torch.cuda.current_stream()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(s)
    fn()
    b.record(s)
    b.synchronize()
    return a.elapsed_time(b)


class Autotuner:
    """best[key] = the fastest configuration measured for that shape key."""

    def __init__(self, reps: int = 2, timer=None):
        self.reps = int(reps)
        self.timer = timer or _cuda_timer
        self.best: dict = {}
        self.trials: dict = {}
        self.tuning_s = 0.0

    def run(self, key, candidates, launch, outputs):
        """launch(outs) runs the operation into the tensors ``outs`` (a list
        shaped like ``outputs``).  The first time ``key`` is seen every
        candidate runs on clones of ``outputs``; then the chosen one runs on
        ``outputs`` themselves."""
        if key not in self.best:
            t0 = time.perf_counter()
            results = []
            for cfg in candidates:
                scratch = [o.clone() for o in outputs]
                with knobs(cfg):
                    launch(scratch)  # warm-up (and first use of any cache)
                    ms = min(self.timer(lambda: launch(scratch)) for _ in range(self.reps))
                results.append((ms, cfg))
            results.sort(key=lambda r: r[0])
            self.best[key] = results[0][1]
            self.trials[key] = results
            self.tuning_s += time.perf_counter() - t0
        with knobs(self.best[key]):
            launch(outputs)

    def summary(self):
        """{key: (best config, best ms, default ms)} for the tuned shapes."""
        out = {}
        for k, res in self.trials.items():
            default = [ms for ms, cfg in res if cfg in ({}, {SPMM_PPT: 2}, {SELECT_BITS: 12})]
            out[k] = (res[0][1], res[0][0], default[0] if default else None)
        return out
