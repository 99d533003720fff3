"""bench.py's reference arm on a small workload (CPU): one JSON line with
the contract's keys."""
import json
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "o10v40", "--steps", "1",
                        "--warmup", "1"], cwd=REPO, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "iter/s" and d["value"] > 0
    for k in ("metric", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling", "vs_baseline",
              "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["e2e"]["value"] == d["value"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    assert d["config"]["workload"].startswith("o10v40")
    # a small workload fits the time budget: whole iterations, nothing extrapolated
    assert d["extrapolated"] is False and cb["extrapolated"] is False and "whole" in cb["sample"]
    assert abs(d["ms_per_step"] - d["timed_wall_ms_per_step"]) < 1e-9


def test_reference_arm_block_sample_mode():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "o10v40", "--steps", "2",
                        "--warmup", "1", "--ref-steps", "blocks"], cwd=REPO, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][0])
    assert d["extrapolated"] is True and "block" in d["cpu_baseline"]["sample"] and d["value"] > 0


def test_clock_sampler_reads_a_fake_nvidia_smi(tmp_path, monkeypatch):
    """The clocks record of the JSON line: the median SM clock under load,
    the maximum clock, and every throttle reason seen active, read from
    nvidia-smi's CSV stream (a fake nvidia-smi on PATH; no GPU involved)."""
    import time
    sys.path.insert(0, REPO)
    import bench
    fake = tmp_path / "nvidia-smi"
    fake.write_text("#!/bin/sh\n"
                    "echo '2070, 2070, 900.5, Not Active, Not Active, Not Active, Not Active'\n"
                    "echo '1980, 2070, 1350.0, Not Active, Not Active, Not Active, Active'\n"
                    "echo '2055, 2070, 1200.0, Not Active, Not Active, Not Active, Not Active'\n"
                    "echo 'garbage line'\n"
                    "exec sleep 30\n")
    fake.chmod(0o755)
    monkeypatch.setenv("PATH", f"{tmp_path}{os.pathsep}{os.environ['PATH']}")
    with bench.ClockSampler(0) as cs:
        t0 = time.time()
        while len(cs.rows) < 3 and time.time() - t0 < 20:
            time.sleep(0.05)
    s = cs.summary()
    assert s == {"sm_mhz": 2055.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    assert bench.ClockSampler(0).summary()["reasons"] == ["unsampled"]


def test_measured_peaks_file_or_fallback():
    sys.path.insert(0, REPO)
    import bench
    p = bench.measured_peaks()
    assert p["hbm_gbs"] > 1000 and p["bf16_tflops"] > 100
    if not os.path.exists(os.path.join(REPO, "MEASURED_PEAKS.json")):
        assert p.get("fallback") is True


def test_peaks_probe_builds():
    """The probe that measures the FP64 and FP32 FMA rates bench.py's roofline
    divides by (python -m fricc_gb300.peaks) cross-compiles for sm_103a."""
    import shutil

    import pytest
    if shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"):
        pytest.skip("nvcc not found")
    sys.path.insert(0, REPO)
    from fricc_gb300 import peaks
    exe = peaks.build()
    assert os.path.exists(exe) and os.access(exe, os.X_OK)


def test_reference_arm_under_torchrun_two_ranks():
    """Launched the way the multi-GPU runs launch bench.py (torchrun, two
    ranks): rank 0 alone runs the reference arm and prints one line; the
    other rank exits 0 without work."""
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
                        "--workload", "o10v40", "--gpus", "2", "--steps", "1", "--warmup", "1"],
                       cwd=REPO, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0


def test_block_plan_covers_every_pair_once():
    """The reference arm's rotating blocks: n_blocks consecutive steps time
    every outer pair of a term exactly once."""
    sys.path.insert(0, REPO)
    import bench
    for n in (1, 7, 400, 900, 4500):
        for nb in (1, 3, 10):
            seen = []
            for b in range(nb):
                (lo, hi), k = bench.block_plan(n, nb, b)
                assert k == hi - lo
                seen.extend(range(lo, hi))
            assert seen == list(range(n))
    assert [bench.n_blocks_for(k) for k in (1, 2, 5, 7, 20, 30)] == [1, 2, 5, 7, 10, 10]


def test_served_sample_parses_the_server_line_and_survives_failure(monkeypatch):
    """bench.py's served_form: the child serve_bench line becomes solves/s,
    p50/p99, the plain FP64 rate, the speed-up and the largest |dE|; a
    failing child is reported as an error, never raised."""
    sys.path.insert(0, REPO)
    import bench

    line = {"served": {"solves_per_s": 15.0, "p50_s": 3.0, "p99_s": 7.5, "converged": 150, "n": 150},
            "plain": {"solves_per_s": 1.25}, "speedup_solves_per_s": 12.0, "max_abs_dE_vs_plain": 4e-7}

    class R:
        def __init__(self, rc, out, err=""):
            self.returncode, self.stdout, self.stderr = rc, out, err

    monkeypatch.setattr(bench.subprocess, "run", lambda *a, **k: R(0, "noise\n" + json.dumps(line) + "\n"))
    d = bench.served_sample(150)
    assert d["solves_per_s"] == 15.0 and d["plain_fp64_solves_per_s"] == 1.25 and d["speedup_vs_plain_fp64"] == 12.0
    assert d["p50_s"] == 3.0 and d["p99_s"] == 7.5 and d["max_abs_dE_vs_plain_fp64"] == 4e-7 and d["requests"] == 150
    monkeypatch.setattr(bench.subprocess, "run", lambda *a, **k: R(1, "", "no device"))
    assert "error" in bench.served_sample(150)
