"""Generate the golden fixtures in this directory from the reference itself.

Runs the reference's own C sources (compiled by ``oracle/Makefile`` target
``ref`` with the single-rank MPI and FFTW stand-ins; needs the reference
source tree, so this script runs only where it is mounted) and records, per
case, the initial and final state in the reference's array layouts, the
explicit RK sources, dt / scheme / time after the run, and the reference's
own log quantities (src/logging.c) where they are printed with full
precision.

Usage:  python tests/golden/make_golden.py      (from the repository root)

Also copies the NPY files the reference's save() writes after a run
(``save_<case>/``) and those its statistics_output() writes after collecting
every step (``stat_<case>/``): the byte-level references for checkpoints and
statistics.

The fixtures are consumed by tests/test_oracle_pinning.py (the C restatement
against them, on the CPU) and tests/test_gpu_plain_parity.py (the CUDA path
against them, on the GPU).
"""
from __future__ import annotations

import json
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.bindings import Config, RefCase, parse_ref_log  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

# name -> (config, expimp cost table w[2*y + x], steps, seeded initial fields?)
CASES = {
    # the 128x256 / Ra=1e8 / Pr=1 Rayleigh-Benard physics on a reduced grid
    "rb_uniform_32x64": (Config(32, 64, Ra=1e8, Pr=1.0), [1.0, 2.0, 2.0, 3.0], 25, False),
    # all four diffusive treatments on a stretched (clipped Chebyshev) grid
    "stretched_expexp": (Config(16, 32, Ra=1e4, Pr=2.0, stretch=3), [1.0, 2.0, 2.0, 3.0], 15, False),
    "stretched_impx": (Config(16, 32, Ra=1e4, Pr=2.0, stretch=3), [3.0, 1.0, 4.0, 5.0], 15, False),
    "stretched_impy": (Config(16, 32, Ra=1e4, Pr=2.0, stretch=3), [3.0, 4.0, 1.0, 5.0], 15, False),
    "stretched_impimp": (Config(16, 32, Ra=1e4, Pr=2.0, stretch=3), [4.0, 3.0, 2.0, 1.0], 15, False),
    # buoyancy switched off, non-square cells, jtot < itot
    "noforcing_24x16": (Config(24, 16, Ra=1e5, Pr=0.7, stretch=2, with_thermal_forcing=False),
                        [1.0, 2.0, 2.0, 3.0], 10, False),
    # arbitrary (seeded) velocity, pressure and temperature fields, no temperature coupling
    "seeded_notemp_32x32": (Config(32, 32, ly=1.0, Ra=1e6, Pr=7.0, with_temperature=False),
                            [1.0, 2.0, 2.0, 3.0], 8, True),
    "seeded_impimp_32x16": (Config(32, 16, ly=0.5, Ra=1e3, Pr=0.7, stretch=5),
                            [4.0, 3.0, 2.0, 1.0], 6, True),
}


def seeded_fields(cfg: Config, seed: int):
    rng = np.random.default_rng(seed)
    su, sc = (cfg.jtot + 2, cfg.itot + 1), (cfg.jtot + 2, cfg.itot + 2)
    ux = 0.1 * rng.uniform(-1, 1, su)
    uy = 0.1 * rng.uniform(-1, 1, sc)
    p = 0.01 * rng.uniform(-1, 1, sc)
    t = rng.uniform(-0.5, 0.5, sc)
    return ux, uy, p, t


# checkpoint fixtures: the reference's own save() output after `steps` steps
SAVE_CASES = {"rb_uniform_32x64": 25}


def save_fixtures():
    import glob
    import shutil

    for name, steps in SAVE_CASES.items():
        cfg, costs, _, _ = CASES[name]
        out = os.path.join(OUT, f"save_{name}")
        shutil.rmtree(out, ignore_errors=True)
        os.makedirs(out)
        with RefCase(cfg) as ref, tempfile.TemporaryDirectory() as d:
            ref.set_costs(costs)
            ref.run(steps)
            if ref.save(d) != 0:
                raise RuntimeError("reference save failed")
            (step_dir,) = glob.glob(os.path.join(d, "output", "save", "step*"))
            for f in sorted(os.listdir(step_dir)):
                shutil.copy(os.path.join(step_dir, f), out)
        print("save", name, sorted(os.listdir(out)))
        # statistics collected after every step (src/statistics/collect.c) and
        # written by statistics_output (src/statistics/output.c)
        out = os.path.join(OUT, f"stat_{name}")
        shutil.rmtree(out, ignore_errors=True)
        os.makedirs(out)
        with RefCase(cfg) as ref, tempfile.TemporaryDirectory() as d:
            ref.set_costs(costs)
            if ref.stats_run(steps, d) != 0:
                raise RuntimeError("reference statistics failed")
            (step_dir,) = glob.glob(os.path.join(d, "output", "stat", "step*"))
            for f in sorted(os.listdir(step_dir)):
                shutil.copy(os.path.join(step_dir, f), out)
        print("stat", name, sorted(os.listdir(out)))


def main():
    save_fixtures()
    manifest = {}
    for seed, (name, (cfg, costs, steps, seeded)) in enumerate(sorted(CASES.items())):
        with RefCase(cfg) as ref:
            ref.set_costs(costs)
            if seeded:
                ref.set_state(*seeded_fields(cfg, 1000 + seed))
            init = ref.get_state()
            ref.run(steps)
            final = ref.get_state()
            src = ref.get_sources()
            dt = ref.get_dt()
            grid = ref.get_grid()
            with tempfile.TemporaryDirectory() as d:
                ref.logging(d)
                log = parse_ref_log(d)
        arrays = {f"init_{k}": v for k, v in init.items() if k != "psi"}
        arrays.update({f"final_{k}": v for k, v in final.items()})
        arrays.update(src)
        arrays.update({f"grid_{k}": np.asarray(v) for k, v in grid.items()})
        arrays["log"] = log
        np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **arrays)
        manifest[name] = {"config": cfg.__dict__, "costs": costs, "steps": steps, "seeded": seeded,
                          "after": dt}
        print(name, dt)
    with open(os.path.join(OUT, "manifest.json"), "w") as fh:
        json.dump(manifest, fh, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
