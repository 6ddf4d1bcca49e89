"""Builds and runs the FP64 pipe probes of this directory on cuda:0.

  fp64_rate.cu  : issue rate of DFMA, DADD, DMUL, DDIV (IEEE), FFMA and IMAD with
                  independent chains (the FP64 denominator of the rooflines)
  fp64_lanes.cu : cost of an FP64 warp instruction versus active lanes and
                  warps per SM, with dependent chains like a Thomas sweep

Usage: python -m simplenavierstokessolver_gb300.probes.run [out_dir]
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def run(out_dir: str = ".") -> dict:
    from simplenavierstokessolver_gb300.build import ARCH, cuda_home

    nvcc = os.path.join(cuda_home(), "bin", "nvcc")
    os.makedirs(out_dir, exist_ok=True)
    logs = {}
    for name in ("fp64_rate", "fp64_lanes"):
        exe = os.path.join(out_dir, name)
        subprocess.run([nvcc, *ARCH, "-O3", "-o", exe, os.path.join(HERE, name + ".cu")], check=True)
        r = subprocess.run([exe], capture_output=True, text=True, check=True)
        logs[name] = r.stdout
        print(r.stdout)
    return logs


if __name__ == "__main__":
    run(sys.argv[1] if len(sys.argv) > 1 else ".")
