"""The tensor-core GEMM's upper-triangle tile schedule, checked on the host:
tests/native/tri_schedule_check.cu compiles the schedule's own functions
(fricc_gb300/csrc/gemm_tc.cu, host-callable) with nvcc, links the library
for the rest of that file, and checks the enumeration against tile_coords
and that the (vv|vv) rebuild's triangle writes every output element once."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def test_triangle_schedule_and_write_once(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    lib = os.path.join(REPO, "fricc_gb300", "_lib", "libfricc_gb300.so")
    if nvcc is None or not os.path.exists(lib):
        pytest.skip("needs nvcc and the built library")
    exe = str(tmp_path / "tri_check")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17",
                    "--expt-relaxed-constexpr", "-o", exe, os.path.join(HERE, "native", "tri_schedule_check.cu"),
                    lib, "-lcuda", f"-Xlinker=-rpath={os.path.dirname(lib)}"], check=True, capture_output=True,
                   timeout=600)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:]
    assert "OK" in r.stdout
