"""The autotuner's choice and replay logic, with a fake timer (no GPU)."""
import pytest

from fricc_gb300 import autotune as AT


class FakeOut:
    def __init__(self):
        self.writes = 0

    def clone(self):
        return FakeOut()


def test_picks_fastest_and_replays(monkeypatch):
    seen = []
    monkeypatch.setattr(AT, "knobs", lambda cfg: _Ctx(seen, cfg))
    cost = {1: 3.0, 2: 1.0, 4: 2.0}
    current = {}

    def timer(fn):
        fn()
        return cost[current["ppt"]]

    tuner = AT.Autotuner(reps=2, timer=timer)
    out = FakeOut()
    launches = []

    def launch(outs):
        launches.append((current.get("ppt"), outs[0] is out))

    _Ctx.current = current
    tuner.run("k", AT.SPMM_CANDIDATES, launch, [out])
    assert tuner.best["k"] == {AT.SPMM_PPT: 2}
    # every candidate ran on scratch (warm-up + 2 timed), then the chosen one on the real output
    assert launches[-1] == (2, True) and sum(1 for _, real in launches if real) == 1
    assert len(launches) == len(AT.SPMM_CANDIDATES) * 3 + 1
    n = len(launches)
    tuner.run("k", AT.SPMM_CANDIDATES, launch, [out])  # replay: one launch, no timing
    assert launches[n:] == [(2, True)]
    s = tuner.summary()
    assert s["k"][0] == {AT.SPMM_PPT: 2} and s["k"][1] == 1.0 and s["k"][2] == 1.0


class _Ctx:
    current = None

    def __init__(self, seen, cfg):
        self.cfg = cfg
        seen.append(cfg)

    def __enter__(self):
        _Ctx.current["ppt"] = self.cfg.get(AT.SPMM_PPT, 2)

    def __exit__(self, *a):
        _Ctx.current.pop("ppt", None)


def test_candidate_sets():
    assert {tuple(sorted(c.items())) for c in AT.SPMM_CANDIDATES} == {((0, 1),), ((0, 2),), ((0, 4),), ((0, 1), (5, 8)),
                                                                     ((0, 2), (5, 8))}
    assert AT.GEMM_CANDIDATES[0] == {} and len(AT.GEMM_CANDIDATES) == 16
    assert [c[AT.SELECT_BITS] for c in AT.COMPRESS_CANDIDATES] == [10, 11, 12, 13]


def test_tune_set_checks_arguments():
    from fricc_gb300 import _lib as L
    lib = L.load()
    assert lib.fricc_tune_set(0, 4) == 0 and lib.fricc_tune_set(0, -1) == 0
    assert lib.fricc_tune_set(0, 3) == 1   # pairs per thread: 1, 2 or 4
    assert lib.fricc_tune_set(1, 5) == 1   # five tiles, 0..4
    assert lib.fricc_tune_set(5, 8) == 0 and lib.fricc_tune_set(5, -1) == 0
    assert lib.fricc_tune_set(5, 9) == 1 and lib.fricc_tune_set(5, 0) == 1   # persistent: 1..8 CTAs per SM
    assert lib.fricc_tune_set(2, 17) == 1  # cover 1..16
    assert lib.fricc_tune_set(3, 0) == 1   # the test-only wait: 1..2^20 polls
    assert lib.fricc_tune_set(3, 1 << 21) == 1
    assert lib.fricc_tune_set(3, 5) == 0 and lib.fricc_tune_set(3, -1) == 0
    assert lib.fricc_tune_set(4, 9) == 1 and lib.fricc_tune_set(4, 14) == 1   # select digit: 10..13 bits
    assert lib.fricc_tune_set(4, 13) == 0 and lib.fricc_tune_set(4, -1) == 0
    assert lib.fricc_tune_set(6, 1) == 1   # no such knob
    assert lib.fricc_tune_set(1, 4) == 0 and lib.fricc_tune_set(1, -1) == 0
