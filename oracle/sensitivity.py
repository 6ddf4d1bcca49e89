"""TEST INFRASTRUCTURE ONLY -- how far rounding-level changes carry in the
FP64 Rayleigh-Benard runs, measured with the CPU oracle alone.

Two experiments, each against the unperturbed oracle run from the
reference's initial condition (srand(0) noise, cost table 1, 2, 2, 3):

  ulp         the temperature interior raised by one ulp at step 0, then
              the same arithmetic (a single perturbation, then amplified by
              the flow);
  contracted  every operation of every step evaluated with fused
              multiply-add contraction (build/liboracle_fma.so: a
              reformulated FP64 path that differs from the reference by
              rounding in every step, as the parallel form of the GPU path
              does).

Prints one JSON line per checkpoint: relative L2 per field (ux, uy, p, T
interiors) after that many steps. These figures set how much reformulation
the 1e-12 bar after the stated step counts allows.

    python oracle/sensitivity.py 512 1024 1e9 2000 --every 250 [--experiment ulp|contracted]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import oracle.bindings as B  # noqa: E402


class ContractedCase(B.OracleCase):
    """the oracle built with contraction (its own library handle)"""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            saved = B.LIBORACLE
            B.LIBORACLE = os.path.join(HERE, "build", "liboracle_fma.so")
            try:
                lib = B.OracleCase.lib.__func__(cls)
            finally:
                B.LIBORACLE = saved
            cls._lib = lib
        return cls._lib


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("nx", type=int)
    ap.add_argument("ny", type=int)
    ap.add_argument("Ra", type=float)
    ap.add_argument("steps", type=int)
    ap.add_argument("--every", type=int, default=250)
    ap.add_argument("--experiment", choices=["ulp", "contracted"], default="ulp")
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    targets = ["liboracle"] + (["contracted"] if args.experiment == "contracted" else [])
    subprocess.run(["make", "-C", HERE, "-s"] + targets, check=True)
    cfg = B.Config(args.nx, args.ny, ly=2.0, Ra=args.Ra, Pr=1.0)
    a = B.OracleCase(cfg, threads=args.threads)
    a.set_costs([1, 2, 2, 3])
    if args.experiment == "contracted":
        b = ContractedCase(cfg, threads=args.threads)
        b.set_costs([1, 2, 2, 3])
    else:
        b = B.OracleCase(cfg, threads=args.threads)
        b.set_costs([1, 2, 2, 3])
        s = b.get_state()
        t = s["temp"].copy()
        t[1:-1, 1:-1] = np.nextafter(t[1:-1, 1:-1], np.inf)
        b.set_state(s["ux"], s["uy"], s["p"], t)
        b.call("update_boundaries")
    marks = sorted(set(list(range(args.every, args.steps, args.every)) + [1, args.steps]))
    done, t0 = 0, time.time()
    for m in marks:
        a.run(m - done)
        b.run(m - done)
        done = m
        sa, sb = a.get_state(), b.get_state()
        row = {"experiment": args.experiment, "step": m}
        for k in ("ux", "uy", "p", "temp"):
            ra, rb = sa[k][1:-1, 1:-1], sb[k][1:-1, 1:-1]
            row[k] = float(np.linalg.norm(ra - rb) / np.linalg.norm(ra))
        row["wall_s"] = round(time.time() - t0, 1)
        print(json.dumps(row), flush=True)


if __name__ == "__main__":
    main()
