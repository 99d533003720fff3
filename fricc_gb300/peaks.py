"""Arithmetic peaks behind the library's roofline figures
(``python -m fricc_gb300.peaks``): builds ``peaks.cu`` for sm_103a into the
package's build folder, runs it on GPU 0 and prints its JSON lines -- the
FP64 FMA rate (denominator of the FP64 contraction kernel), the FP32 FMA
rate (÷ 12 instructions per FP32-pair multiply-add × 2 flops: denominator of
the FP32-pair kernels), FP64 mma.sync and a plain copy for scale.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys

from . import build as B

SRC = os.path.join(os.path.dirname(os.path.abspath(__file__)), "peaks.cu")
EXE = os.path.join(B.LIBDIR, "peaks")


def build() -> str:
    os.makedirs(B.LIBDIR, exist_ok=True)
    if B._stale(EXE, [SRC]):
        r = subprocess.run([B.nvcc(), *B.ARCH, "-O3", "-std=c++17", "-lineinfo", SRC, "-o", EXE],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on peaks.cu\n{r.stdout}\n{r.stderr}")
    return EXE


def run() -> list:
    r = subprocess.run([build()], capture_output=True, text=True, timeout=600)
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    if r.returncode != 0:
        raise RuntimeError(f"peaks failed ({r.returncode}): {r.stdout[-2000:]} {r.stderr[-2000:]}")
    return lines


if __name__ == "__main__":
    for line in run():
        print(json.dumps(line))
    sys.exit(0)
