"""Measure the arithmetic peaks the library's kernels are bounded by.

Builds csrc/probes/peaks.cu for sm_103a, runs it on device 0 and writes the
result to profiles/fp64_peak.json (FP64 DFMA / DMMA and legacy bf16 mma.sync
throughput).  The measured HBM and cuBLAS bf16 peaks live in
MEASURED_PEAKS.json; this file adds the FP64 figure those do not cover.

Usage: python -m itg.peaks   (from itensorsgpu.jl_gb300/, on a GPU machine)
"""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

from .build import ARCH_FLAGS, BUILD_DIR, CSRC, REPO, _nvcc


def build_probe() -> Path:
    BUILD_DIR.mkdir(exist_ok=True)
    exe = BUILD_DIR / "peaks"
    src = CSRC / "probes" / "peaks.cu"
    if not exe.exists() or exe.stat().st_mtime < src.stat().st_mtime:
        subprocess.run([_nvcc(), *ARCH_FLAGS, "-O3", "-std=c++17", str(src), "-o", str(exe)], check=True)
    return exe


def main():
    exe = build_probe()
    r = subprocess.run([str(exe)], capture_output=True, text=True, check=True)
    data = json.loads(r.stdout.strip().splitlines()[-1])
    data["fp64_tflops"] = max(data["fp64_dfma_tflops"], data["fp64_dmma_tflops"])
    out = REPO / "profiles" / "fp64_peak.json"
    out.parent.mkdir(exist_ok=True)
    out.write_text(json.dumps(data, indent=1) + "\n")
    print(json.dumps(data))


if __name__ == "__main__":
    sys.exit(main())
