"""Benchmark of the SMR-RK3 time step on GB300.

Workload (default): 2D Rayleigh-Benard, 512 x 1024 uniform staggered grid,
lx = 1, ly = 2, Ra = 1e9, Pr = 1, u = p = 0 and T = linear profile + uniform
noise in [-0.05, 0.05] (the reference's own initial condition), dt and the
explicit/implicit choice from param_decide_dt every step. One bench "step" is
one solver time step: the device max-|u| reduction and dt decision plus the
three RK substages (temperature, momentum, Poisson, projection, pressure).

Arms:
  default          the plain FP64 GPU path of libsns_gpu.so in the form --form
                   names (default parallel: partition-method line solves and
                   radix-8 DFTs, within 1e-12 of the reference; exact: the
                   reference's operations, bit-identical), the other form's
                   figure beside it; inputs resident in HBM; per-step CUDA
                   events on the solver's stream; L2 flushed (256 MiB write)
                   between timed steps.
  --impl reference the CPU oracle (the reference's algorithm restated in C, bit
                   identical to it) on all host cores, same workload and metric.

The JSON line also carries the per-kernel roofline of the dominant kernel
(CUDA events around each launch, a second pass of the same steps) against
HBM and against the FP64 issue rate measured in the run, the CPU baseline,
an end-to-end number through the C ABI with host buffers, kernel launch
counts and the SM clocks sampled during the timed region; beyond the
headline, the batched FP32 and compensated forms (one case, the 64-case
ensemble, with accuracy against FP64), the serving stream and the
2048 x 4096 instance over 500 steps (--plain-only, --large-only and
--serving-only run parts alone).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PEAKS_PATH = os.path.join(ROOT, "MEASURED_PEAKS.json")
METRIC = "cell-steps/s plain FP64 vs batched FP32-stencil at stated L2 error; p50/p99"
FALLBACK_HBM_GBS = 6800.0

# algorithmic DRAM bytes per cell per launch (FP64, explicit scheme) and FP64
# instructions per cell, per kernel, from the kernels' loads/stores and
# arithmetic (beta != 0 substages; rk=0 skips one 8-byte read and two FP64 ops)
KERNEL_MODEL = {
    # name: (bytes per cell, fp64 ops per cell)
    "temperature_update": (48.0, 27.0),
    "velocity_update": (80.0, 81.0),
    # on grids whose spacings are powers of two, 29 of the 81 products (the 1/2
    # weights, reciprocal spacings, advective coefficients) run in the integer unit
    "velocity_update_p2": (80.0, 52.0),
    "poisson_forward_fft": (24.0, None),
    "poisson_tridiagonal": (40.0, 5.0),
    # partition-method solve of the parallel form: the spectrum read and
    # written once (its RHS-independent factor blocks stay in L2)
    "poisson_pcr": (16.0, None),
    "poisson_inverse_fft": (16.0, None),
    "correct_and_pressure": (56.0, 9.0),
    "max_velocity": (16.0, 0.0),
    # forward DFT + tridiagonal + inverse DFT + explicit temperature update in
    # one launch. Compulsory bytes of the Poisson solve: read ux*, uy* (16),
    # write the spectrum (8), read and write it in the tridiagonal solve (16),
    # read it in the inverse DFT (8), write psi (8) = 56; the temperature
    # update 48. The Thomas factors (RHS-independent, precomputed) are not
    # counted: they stay in L2 between launches.
    "poisson_fused": (56.0 + 48.0, None),
}


# DRAM bytes (read + write) per launch from ncu captures of the default
# workload, keyed by kernel and size: the fused launch from
# profiles/plain_fp64_fused_512x1024_ncu.md; the velocity update (16.8-25.2 MB
# per launch in either form; the larger figure is used) and the parallel
# form's kernels from profiles/plain_parallel_fp64_counts_512x1024.md; the
# exact form's three-kernel Poisson solve from an earlier capture of the same
# size
PROFILED_TRAFFIC = {
    ("poisson_fused", 512, 1024): 29699840 + 19200,  # profiles/plain_fp64_fused_512x1024_ncu.md
    ("poisson_tridiagonal", 512, 1024): 8665344,
    ("velocity_update", 512, 1024): 25210880,
    ("poisson_forward_fft", 512, 1024): 8440064,
    ("temperature_update", 512, 1024): 12647168,
    ("poisson_inverse_fft", 512, 1024): 4249088,
    ("correct_and_pressure", 512, 1024): 16805376,
}


# FP64 instructions per cell of the parallel form's kernels on a uniform
# power-of-two grid (DADD + DMUL + DFMA thread instructions counted by ncu at
# 512 x 1024: profiles/plain_parallel_fp64_counts_512x1024.md; the temperature
# update's mean over the three substages, the first of which has no previous
# source; the DFT counts grow with log2(jtot))
PARALLEL_FP64_OPS = {"velocity_update": 47.45, "temperature_update": 17.17, "poisson_forward_fft": 20.63,
                     "poisson_pcr": 5.39, "poisson_inverse_fft": 17.75, "correct_and_pressure": 9.0}

# algorithmic DRAM bytes per cell of the plain path's implicit-scheme
# launches (2048 x 4096 at Ra 1e10): each Crank-Nicolson launch solves the
# temperature, ux and uy lines side by side (increment read and written per
# field), the increment launch adds them to the three fields
IMPLICIT_MODEL = {"cn_solve_x": 48.0, "cn_solve_y": 48.0, "add_increment": 72.0}


def batched_bytes_per_cell_step(compensated: bool) -> float:
    """algorithmic DRAM bytes per cell and time step of the batched form:
    per substage the stencil (hi and lo words of ux, uy, T read and written,
    24 + 24 B; previous right-hand sides 12 + 12 B, their low words too when
    compensated; p 8 B), the divergence and forward DFT (ux, uy pairs 16 B,
    half-spectrum 8 B), the tridiagonal solve (spectrum 8 + 8 B, factors
    16 B), the inverse DFT (8 + 8 B) and the correction (psi, p 16 B, the
    velocity pairs 16 + 16 B, p 8 B)"""
    stencil = 80.0 + (24.0 if compensated else 0.0)
    return 3 * (stencil + 24.0 + 32.0 + 16.0 + 56.0)


def power_of_two_grid(grid: dict) -> bool:
    """every spacing a power of two 2^e, |e| <= 64: the velocity kernel then
    forms its power-of-two products in integer arithmetic"""
    import math

    def p2(v):
        m, e = math.frexp(float(v))
        return v > 0 and m == 0.5 and abs(e - 1) <= 60

    return p2(grid["dy"]) and all(p2(v) for v in grid["dxf"]) and all(p2(v) for v in grid["dxc"])


def fft_ops_per_cell(ny: int, forward: bool) -> float:
    """FP64 instructions per real sample of one length-ny real FFT as the
    kernels perform it (radix-2 first stage if log2(ny/2) is odd, radix-4
    stages with twiddles after the first, split step), plus the divergence
    (forward) or the 1/ny scaling (inverse)."""
    m = ny // 2
    p = m.bit_length() - 1
    stages = ([2] if p % 2 else []) + [4] * (p // 2)
    ops, L = 0.0, 1
    for s, r in enumerate(stages):
        nb = m // r
        per = (4 if r == 2 else 16) + ((r - 1) * 6 if L > 1 else 0)
        ops += nb * per
        L *= r
    ops += (m // 2) * 18 + 2  # split step pairs
    per_sample = ops / ny
    return per_sample + (6.0 if forward else 1.0)


def load_peaks():
    try:
        with open(PEAKS_PATH) as fh:
            pk = json.load(fh)
        return float(pk["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms, each sample
    stamped with the host clock so that those inside a timed region can be
    told apart (`mark`)."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.thread = None
        self.region = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def mark(self, t0: float, t1: float):
        """the timed region, in time.perf_counter() seconds"""
        self.region = (t0, t1)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons, power, inside = [], [], set(), [], []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for t, ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            # a sample printed within 50 ms after the region's end was taken in it
            if self.region and self.region[0] <= t <= self.region[1] + 0.05:
                inside.append(sm[-1])
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(inside or sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm), "samples_in_timed_region": len(inside),
                "sm_mhz_timed_region": statistics.median(inside) if inside else None,
                "power_w_max": max(power) if power else None,
                "window": "from before the warm-up to after the per-kernel pass (the same steps replayed)"}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo", init_method="env://")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(value: float, world: int) -> float:
    if world == 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ----------------------------------------------------------------- CPU arms
def cpu_oracle_rate(cfg, seconds: float, threads: int, min_steps: int = 2):
    """cell-steps/s of the CPU oracle on a bounded sample of the workload"""
    from oracle.bindings import OracleCase

    o = OracleCase(cfg, threads=threads)
    o.run(1)  # warm-up (page-in, first-touch)
    n, t0 = 0, time.perf_counter()
    while n < min_steps or time.perf_counter() - t0 < seconds:
        o.run(1)
        n += 1
    el = time.perf_counter() - t0
    o.close()
    return cfg.itot * cfg.jtot * n / el, n, el


def reference_arm(args, world, rank):
    from oracle.build import build as build_oracle
    from oracle.bindings import Config

    if rank != 0:
        return 0
    build_oracle()
    cfg = Config(args.nx, args.ny, ly=2.0, Ra=args.Ra, Pr=args.Pr)
    threads = os.cpu_count() or 1
    from oracle.bindings import OracleCase

    o = OracleCase(cfg, threads=threads)
    for _ in range(args.warmup):
        o.run(1)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        o.run(1)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = cfg.itot * cfg.jtot * args.steps / total
    line = {
        "metric": METRIC, "value": value, "unit": "cell-steps/s",
        "impl": "reference", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (reference initial condition, srand(0))",
        "config": workload_config(args),
        "cpu_baseline": {"value": value, "unit": "cell-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} time steps of {args.nx}x{args.ny} after {args.warmup} warm-up"},
        "e2e": {"value": value, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def workload_config(args):
    return {"workload": f"rayleigh_benard_{args.nx}x{args.ny}_Ra{args.Ra:g}_Pr{args.Pr:g}",
            "nx": args.nx, "ny": args.ny, "lx": 1.0, "ly": 2.0, "Ra": args.Ra, "Pr": args.Pr,
            "grid": "uniform", "scheme": "explicit x / explicit y (chosen by param_decide_dt)",
            "l2": "flushed between timed steps (256 MiB write)", "parallelism": "replicas only"}


# ------------------------------------------------------ FP32-stencil / batched
def fp32_single(args, torch, compensated=False):
    """throughput of the FP32-stencil / FP64-Poisson form on the same case,
    with the launch shapes picked by sns_batch_autotune (the default shapes'
    rate beside it; shapes change speed, not results); compensated: the
    float-float stencil terms and increments"""
    from simplenavierstokessolver_gb300.batch import Batch, Desc

    cells = args.nx * args.ny
    with Batch(8 << 30) as b:
        s = b.add(Desc(args.nx, args.ny, ly=2.0, Ra=args.Ra, Pr=args.Pr, compensated=compensated))
        stream = torch.cuda.ExternalStream(b.stream())
        flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
        b.step(args.warmup)
        b.synchronize()

        def timed():
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                  for _ in range(args.steps)]
            for a, e in ev:
                a.record(stream)
                b.step(1)
                e.record(stream)
                with torch.cuda.stream(stream):
                    flush.zero_()
            b.synchronize()
            return sum(a.elapsed_time(e) for a, e in ev)

        ms_default = timed()
        shapes, _ = b.autotune(steps=5)
        b.step(args.warmup)
        b.synchronize()
        ms = timed()
        del b, s
    value = cells * args.steps / (ms * 1e-3)
    return {"value": value, "unit": "cell-steps/s", "ms_per_step": ms / args.steps,
            "default_shapes_value": cells * args.steps / (ms_default * 1e-3), "autotuned_shapes": shapes,
            "l2": "flushed between timed steps (256 MiB write)", "hbm_roofline": hbm_roofline(value, compensated)}


def hbm_roofline(cell_steps_per_s: float, compensated: bool) -> dict:
    """the batched form's whole step against the measured HBM bandwidth"""
    peak, kind = load_peaks()
    bpc = batched_bytes_per_cell_step(compensated)
    gbs = cell_steps_per_s * bpc / 1e9
    return {"bytes_per_cell_step": bpc, "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
            "peak_source": f"{kind} (MEASURED_PEAKS.json hbm_gbs)" if kind == "measured" else "fallback",
            "note": "algorithmic bytes of the whole step over its event time; the FP64 DFTs bound the step"}


def large_instance(args, torch, nx=2048, ny=4096, Ra=1e10, steps=500, acc_steps=200):
    """The 2048 x 4096, Ra 1e10 instance.

    Plain FP64 in both arithmetic forms: `steps` steps of sns_run (treatment
    by param_decide_dt with the fixed cost table: Crank-Nicolson in x and y
    here), a CUDA event pair around every step on the solver's stream (each
    sns_run call ends with a host synchronisation, so an interval holds the
    step's device work and any host gap inside it), per-kernel times from a
    profiled pass. The FP32 and compensated batched forms integrate
    explicitly (their dt is the explicit limit), so beside cell-steps/s every
    leg reports simulated time per wall second. Accuracy of the two batched
    forms: `acc_steps` steps against the plain FP64 path made to take the
    same explicit steps (the batch's dt sequence replayed)."""
    import ctypes

    import numpy as np

    from simplenavierstokessolver_gb300 import Case
    from simplenavierstokessolver_gb300.batch import Batch, Desc

    cells = nx * ny
    out = {"workload": f"rayleigh_benard_{nx}x{ny}_Ra{Ra:.0e}_Pr1", "steps": steps}
    peak, _ = load_peaks()
    for form in ("exact", "parallel"):
        with Case(nx, ny, ly=2.0, Ra=Ra, Pr=1.0) as c:
            lib = c.lib
            c.set_form(form == "parallel")
            stream = torch.cuda.ExternalStream(c.stream())
            c.run(3)
            c.synchronize()
            t0 = c.get_dt()["time"]
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
            schemes = []
            for a, b in ev:
                a.record(stream)
                c.run(1)
                b.record(stream)
                dd = c.get_dt()
                schemes.append((dd["implicitx"], dd["implicity"]))
            c.synchronize()
            per = np.array([a.elapsed_time(b) for a, b in ev])
            imp = np.array([bool(x or y) for x, y in schemes], dtype=bool)
            ms = float(per.sum())
            d = c.get_dt()
            sim = d["time"] - t0
            lib.sns_profile(c.fluid, 1)
            c.run(2)
            c.synchronize()
            kms = (ctypes.c_double * 32)()
            kcnt = (ctypes.c_longlong * 32)()
            n = lib.sns_profile_read(c.fluid, kms, kcnt, 32)
            lib.sns_profile(c.fluid, 0)
            kernels = {lib.sns_profile_kind_name(k).decode(): round(1e3 * kms[k] / kcnt[k], 1)
                       for k in range(n) if kcnt[k]}
        # per-kernel times of implicit steps (Crank-Nicolson in x and y): the
        # first steps of a fresh case, profiled; the timed run above is not touched
        with Case(nx, ny, ly=2.0, Ra=Ra, Pr=1.0) as c:
            lib = c.lib
            c.set_form(form == "parallel")
            c.run(3)
            lib.sns_profile(c.fluid, 1)
            c.run(2)
            c.synchronize()
            dimp = c.get_dt()
            kms = (ctypes.c_double * 32)()
            kcnt = (ctypes.c_longlong * 32)()
            n = lib.sns_profile_read(c.fluid, kms, kcnt, 32)
            lib.sns_profile(c.fluid, 0)
            kernels_imp = {lib.sns_profile_kind_name(k).decode(): round(1e3 * kms[k] / kcnt[k], 1)
                           for k in range(n) if kcnt[k]}
            scheme_imp = (dimp["implicitx"], dimp["implicity"])
        kgbs = {}
        for k, us in kernels.items():
            bpc = IMPLICIT_MODEL.get(k, KERNEL_MODEL.get(k, (None,))[0])
            if bpc and us > 0:
                gbs = bpc * cells / (us * 1e-6) / 1e9
                kgbs[k] = {"bytes_per_cell": bpc, "achieved_gbs": round(gbs, 1), "frac": round(gbs / peak, 4)}
        out[f"plain_fp64_{form}"] = {
            "value": cells * steps / (ms * 1e-3), "ms_per_step": ms / steps,
            "ms_step_median": float(np.median(per)), "ms_step_min": float(per.min()), "ms_step_max": float(per.max()),
            "simulated_time_per_s": sim / (ms * 1e-3), "simulated_time": sim,
            "scheme": "param_decide_dt per step with the cost table (1, 2, 2, 3): Crank-Nicolson in x and y "
                      "while the explicit diffusive limit is the tighter one, explicit once the flow is fast",
            "implicit_steps": int(imp.sum()), "explicit_steps": int((~imp).sum()),
            "ms_step_implicit_median": float(np.median(per[imp])) if imp.any() else None,
            "ms_step_explicit_median": float(np.median(per[~imp])) if (~imp).any() else None,
            "kernel_avg_us": kernels, "kernel_hbm": kgbs, "hbm_peak_gbs": peak,
            "kernel_avg_us_implicit": {"scheme_xy": list(scheme_imp), "steps": "4 and 5 of a fresh case",
                                       "kernels": kernels_imp}}
    for name, comp in (("fp32_stencil", False), ("fp32_compensated", True)):
        with Batch(16 << 30) as b:
            s = b.add(Desc(nx, ny, ly=2.0, Ra=Ra, Pr=1.0, compensated=comp))
            stream = torch.cuda.ExternalStream(b.stream())
            b.step(3)
            shapes, _ = b.autotune(steps=3)
            b.step(2)
            b.synchronize()
            t0 = b.status(s)["time"]
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            b.step(steps)
            e1.record(stream)
            b.synchronize()
            ms = e0.elapsed_time(e1)
            sim = b.status(s)["time"] - t0
        v32 = cells * steps / (ms * 1e-3)
        out[name] = {"value": v32, "ms_per_step": ms / steps, "simulated_time_per_s": sim / (ms * 1e-3),
                     "scheme": "explicit x / explicit y (batched form)", "autotuned_shapes": shapes,
                     "hbm_roofline": hbm_roofline(v32, comp)}
        if acc_steps > 0:
            out[name]["accuracy_vs_fp64"] = batched_accuracy(nx, ny, Ra, 1.0, acc_steps, comp)
    return out


def batched_accuracy(nx, ny, Ra, Pr, nsteps, compensated):
    from simplenavierstokessolver_gb300.batch import Desc

    return batched_accuracy_desc(Desc(nx, ny, ly=2.0, Ra=Ra, Pr=Pr, compensated=compensated), nsteps)


def batched_accuracy_desc(desc, nsteps):
    """relative L2 per field (p modulo its mean) of a batched-form run of
    `desc` against the plain FP64 path (exact form) taking the same explicit
    steps from the same initial state: the batch's dt sequence replayed"""
    import dataclasses

    import numpy as np

    from simplenavierstokessolver_gb300 import Case
    from simplenavierstokessolver_gb300.batch import Batch, initial_temperature

    desc = dataclasses.replace(desc, steps=0)
    dts = []
    with Batch(16 << 30) as b:
        s = b.add(desc)
        for _ in range(nsteps):
            dts.append(b.status(s)["dt"])
            b.step(1)
        got = b.state(s)
        finite = b.status(s)["finite"]
    with Case(desc.itot, desc.jtot, ly=desc.ly, stretch=desc.stretch, Ra=desc.Ra, Pr=desc.Pr) as c:
        st = c.get_state()
        c.set_state(st["ux"], st["uy"], st["p"], initial_temperature(desc))
        for dt in dts:
            c.set_dt(dt, 0, 0)
            c.integrate()
        c.synchronize()
        ref = c.get_state()
    err = {}
    for k in ("ux", "uy", "temp", "p"):
        a, r = got[k][1:-1, 1:-1], ref[k][1:-1, 1:-1]
        if k == "p":
            a, r = a - a.mean(), r - r.mean()
        err[k] = float(np.linalg.norm(a - r) / np.linalg.norm(r))
    return {"steps": nsteps, "time": float(sum(dts)), "rel_l2": err, "finite": bool(finite),
            "dt": "explicit dt of the batched run, replayed in the FP64 run"}


def fp32_accuracy(args, compensated=False):
    """The FP32-stencil form against the bit-exact FP64 path (identical to the
    reference) over args.acc_steps steps with the same dt sequence: the
    batch's own CFL dt is replayed into the FP64 solver. Returns relative L2
    per field (p modulo its mean) and both sets of Nusselt numbers."""
    import numpy as np

    from simplenavierstokessolver_gb300 import Case
    from simplenavierstokessolver_gb300.batch import Batch, Desc

    nsteps = args.acc_steps
    desc = Desc(args.nx, args.ny, ly=2.0, Ra=args.Ra, Pr=args.Pr, compensated=compensated)
    dts = []
    with Batch(8 << 30) as b:
        s = b.add(desc)
        for _ in range(nsteps):
            dts.append(b.status(s)["dt"])
            b.step(1)
        got = b.state(s)
        diag32 = b.diagnostics(s)
    with Case(args.nx, args.ny, ly=2.0, Ra=args.Ra, Pr=args.Pr) as c:
        for dt in dts:
            c.set_dt(dt, 0, 0)
            c.integrate()
        c.synchronize()
        ref = c.get_state()
        diag64 = c.diagnostics()
    err = {}
    for k in ("ux", "uy", "temp", "p"):
        a, r = got[k][1:-1, 1:-1], ref[k][1:-1, 1:-1]
        if k == "p":
            a, r = a - a.mean(), r - r.mean()
        err[k] = float(np.linalg.norm(a - r) / np.linalg.norm(r))
    names = ["nu_wall", "nu_injection", "nu_kinetic_dissipation", "nu_thermal_dissipation"]
    return {"steps": nsteps, "time": float(sum(dts)), "dt": "CFL dt of the FP32 run, replayed in the FP64 run",
            "rel_l2": err, "nusselt_fp64": dict(zip(names, diag64[7:].tolist())),
            "nusselt_fp32_stencil": dict(zip(names, diag32[7:].tolist())),
            "divergence_max_fp32_stencil": float(diag32[0]), "divergence_max_fp64": float(diag64[0])}


def ensemble_throughput(args, torch, compensated=False):
    """64-case ensemble: batched FP32-stencil form (one graph launch per step
    for all cases, launch shapes picked by sns_batch_autotune; the default
    shapes' rate beside it) against the plain FP64 path stepping the cases
    one by one (compensated: the batched rates only)"""
    from simplenavierstokessolver_gb300 import Case
    from simplenavierstokessolver_gb300.batch import Batch
    from simplenavierstokessolver_gb300.workloads import ensemble

    descs = ensemble(64)
    for d in descs:
        d.compensated = compensated
    cells = sum(d.itot * d.jtot for d in descs)
    with Batch(8 << 30) as b:
        for d in descs:
            b.add(d)
        stream = torch.cuda.ExternalStream(b.stream())
        b.step(args.warmup)
        b.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

        def timed():
            e0.record(stream)
            b.step(args.ens_steps)
            e1.record(stream)
            b.synchronize()
            return e0.elapsed_time(e1)

        default_shapes = b.tuning()
        ms_default = timed()
        tuned_shapes, _ = b.autotune(steps=5)
        ms_b = timed()
        # A/B: one persistent cooperative launch per substage (same shapes,
        # same results) against the step graph of per-phase launches
        persistent = None
        try:
            b.set_persistent(True)
            b.step(args.warmup)
            b.synchronize()
            ms_p = timed()
            persistent = {"value": cells * args.ens_steps / (ms_p * 1e-3), "vs_graph_of_phases": ms_b / ms_p,
                          "launches_per_step": 4}
        except Exception as err:  # noqa: BLE001 -- reported; the per-phase form stands
            persistent = {"unavailable": str(err)}
        finally:
            b.set_persistent(False)
    batched = cells * args.ens_steps / (ms_b * 1e-3)
    batched_default = cells * args.ens_steps / (ms_default * 1e-3)
    if compensated:
        return {"cases": len(descs), "cells": cells, "batched_compensated": batched,
                "batched_default_shapes": batched_default, "autotuned_shapes": tuned_shapes,
                "persistent_substage": persistent,
                "unit": "cell-steps/s", "batched_steps": args.ens_steps,
                "hbm_roofline": hbm_roofline(batched, True)}
    plain_steps = max(2, args.ens_steps // 5)
    total_s, plain_cells = 0.0, 0
    for d in descs:
        with Case(d.itot, d.jtot, ly=d.ly, Ra=d.Ra, Pr=d.Pr) as c:
            c.run(2)
            t0 = time.perf_counter()
            c.run(plain_steps)
            total_s += time.perf_counter() - t0
            plain_cells += d.itot * d.jtot
    plain = plain_cells * plain_steps / total_s
    # the plain path at its best on many small cases: every case on its own
    # stream with its first CFL dt kept fixed (no per-step host decision), the
    # Poisson solve as three kernels (the fused launch takes the whole GPU),
    # steps issued round-robin so that the cases' kernels overlap
    def concurrent(parallel_form):
        cases = [Case(d.itot, d.jtot, ly=d.ly, Ra=d.Ra, Pr=d.Pr) for d in descs]
        try:
            for c in cases:
                c.set_fused(False)
                c.set_form(parallel_form)
                c.param_decide_dt()
                c.integrate()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(plain_steps):
                for c in cases:
                    c.integrate()
            for c in cases:
                c.synchronize()
            return cells * plain_steps / (time.perf_counter() - t0)
        finally:
            for c in cases:
                c.close()

    plain_concurrent_exact = concurrent(False)
    plain_concurrent_parallel = concurrent(True)
    plain_concurrent = max(plain_concurrent_exact, plain_concurrent_parallel)
    return {"cases": len(descs), "cells": cells, "batched_fp32_stencil": batched,
            "batched_default_shapes": batched_default, "default_shapes": default_shapes,
            "autotuned_shapes": tuned_shapes, "persistent_substage": persistent, "plain_fp64_one_by_one": plain,
            "plain_fp64_concurrent_streams": plain_concurrent,
            "plain_fp64_concurrent_streams_exact_form": plain_concurrent_exact,
            "plain_fp64_concurrent_streams_parallel_form": plain_concurrent_parallel,
            "ratio_vs_concurrent": batched / plain_concurrent,
            "ratio": batched / plain, "unit": "cell-steps/s", "batched_steps": args.ens_steps,
            "hbm_roofline": hbm_roofline(batched, False),
            "plain_steps_per_case": plain_steps,
            "workload": "nx in {64,128,256}, ny=2nx, log10 Ra in [6,9], Pr in [0.7,7], SplitMix64 seeds 20261203+k"}


def ensemble_accuracy(args, compensated=False):
    """The 64-case ensemble in the batched FP32-stencil form against the FP64
    path (bit-identical to the reference) over args.ens_acc_steps steps: each
    case starts from its seeded initial temperature in both runs, and the
    batch's CFL dt sequence is replayed into the FP64 run. Relative L2 per
    field over the interior (p modulo its mean); max and median over cases.
    The sensitivity control (FP64 from a perturbed start) runs for the FP32
    form only."""
    import numpy as np

    from simplenavierstokessolver_gb300 import Case
    from simplenavierstokessolver_gb300.batch import Batch, initial_temperature
    from simplenavierstokessolver_gb300.workloads import ensemble

    descs = ensemble(64)
    for d in descs:
        d.compensated = compensated
    n = args.ens_acc_steps
    dts = [[] for _ in descs]
    with Batch(8 << 30) as b:
        slots = [b.add(d) for d in descs]
        for _ in range(n):
            for k, s in enumerate(slots):
                dts[k].append(b.status(s)["dt"])
            b.step(1)
        got = [b.state(s) for s in slots]
    fields = ("ux", "uy", "temp", "p")

    def fp64_run(d, dt_seq, t0):
        with Case(d.itot, d.jtot, ly=d.ly, Ra=d.Ra, Pr=d.Pr) as c:
            st = c.get_state()
            c.set_state(np.zeros_like(st["ux"]), np.zeros_like(st["uy"]), np.zeros_like(st["p"]), t0)
            for dt in dt_seq:
                c.set_dt(dt, 0, 0)
                c.integrate()
            return c.get_state()

    def rel(a_state, r_state):
        out = {}
        for f in fields:
            a, r = a_state[f][1:-1, 1:-1], r_state[f][1:-1, 1:-1]
            if f == "p":
                a, r = a - a.mean(), r - r.mean()
            nr = np.linalg.norm(r)
            out[f] = float(np.linalg.norm(a - r) / nr) if nr > 0 else 0.0
        return out

    # sensitivity control: the FP64 path itself, started from T perturbed by
    # a relative 1e-9 (seeded), after the same steps; growth = error / 1e-9
    eps = 1e-9
    rng = np.random.default_rng(20261203)
    errs, growth = [], []
    for k, d in enumerate(descs):
        t0 = initial_temperature(d)
        ref = fp64_run(d, dts[k], t0)
        errs.append(rel(got[k], ref))
        if compensated:
            continue
        tp = t0.copy()
        tp[1:-1, 1:-1] *= 1.0 + eps * rng.uniform(-1.0, 1.0, tp[1:-1, 1:-1].shape)
        growth.append(max(rel(fp64_run(d, dts[k], tp), ref).values()) / eps)
    worst = [max(e.values()) for e in errs]
    within = [w <= 1e-5 for w in worst]
    if compensated:
        return {"steps": n, "dt": "CFL dt of the compensated run, replayed in the FP64 run",
                "rel_l2_max": {f: max(e[f] for e in errs) for f in fields},
                "rel_l2_median": {f: float(np.median([e[f] for e in errs])) for f in fields},
                "target": 1e-5, "cases_within_target": int(sum(within)),
                "worst_case": {"nx": descs[int(np.argmax(worst))].itot, "Ra": descs[int(np.argmax(worst))].Ra,
                               "rel_l2_max": max(worst)}}
    outside = [{"nx": descs[k].itot, "Ra": descs[k].Ra, "Pr": descs[k].Pr, "rel_l2_max": worst[k],
                "fp64_growth_of_1e-9": growth[k]} for k in range(len(descs)) if not within[k]]
    return {"steps": n, "dt": "CFL dt of the FP32 run, replayed in the FP64 run",
            "rel_l2_max": {f: max(e[f] for e in errs) for f in fields},
            "rel_l2_median": {f: float(np.median([e[f] for e in errs])) for f in fields},
            "target": 1e-5, "cases_within_target": int(sum(within)),
            "fp64_growth_of_1e-9_median": float(np.median(growth)),
            "cases_outside_target": sorted(outside, key=lambda o: -o["rel_l2_max"])}


def serving(args):
    """sns_serve on a Poisson stream of requests: time to completion and queue
    wait percentiles, aggregate cell-steps/s over the busy span, the number of
    requests whose final state holds a NaN or infinity, and for a seeded
    sample of requests (the cheapest few) the relative L2 error of the served
    result against the plain FP64 path taking the same explicit steps (a
    request's arithmetic reads only its own data, so its result served alone
    equals its result in the mix: tests/test_gpu_batch.py)"""
    import dataclasses

    import numpy as np

    from simplenavierstokessolver_gb300.batch import serve
    from simplenavierstokessolver_gb300.workloads import serving_stream

    descs, arrivals = serving_stream(args.serve_rate, args.serve_seconds)
    descs = [dataclasses.replace(d, compensated=args.serve_compensated) for d in descs]
    r = serve(descs, arrivals, hbm_bytes=args.serve_hbm << 20, max_cases=256, chunk_steps=args.serve_chunk)
    arr = np.asarray(arrivals)
    ttc = r["done"] - arr
    wait = r["admit"] - arr
    work = sum(d.itot * d.jtot * d.steps for d in descs)
    out = {"requests": len(descs), "rate_per_s": args.serve_rate, "arrival_window_s": args.serve_seconds,
           "form": "compensated (float-float stencils)" if args.serve_compensated else "FP32 stencils",
           "p50_s": float(np.percentile(ttc, 50)), "p99_s": float(np.percentile(ttc, 99)),
           "queue_wait_p50_s": float(np.percentile(wait, 50)), "queue_wait_p99_s": float(np.percentile(wait, 99)),
           "mean_queue_wait_s": float(np.mean(wait)),
           "value": work / r["busy_s"], "unit": "cell-steps/s", "busy_s": r["busy_s"],
           "nonfinite_requests": int((~r["finite"]).sum()),
           "hbm_arena_bytes": args.serve_hbm << 20, "chunk_steps": args.serve_chunk,
           "workload": "Poisson arrivals; nx in {64,128,256,512}, ny=2nx, log10 Ra in [6,10], Pr in [0.7,7], "
                       "steps in {200..2000}"}
    if args.serve_acc_sample > 0:
        order = sorted(range(len(descs)), key=lambda k: descs[k].itot * descs[k].jtot * descs[k].steps)
        sample = order[:args.serve_acc_sample]
        out["accuracy_sample"] = [
            {"request": k, "nx": descs[k].itot, "Ra": descs[k].Ra, "Pr": descs[k].Pr, "steps": descs[k].steps,
             **batched_accuracy_desc(descs[k], descs[k].steps)} for k in sample]
    return out


# ----------------------------------------------------------------- GPU arm
def gpu_arm(args, world, rank, local):
    import torch

    from simplenavierstokessolver_gb300.build import build as build_lib

    build_lib()
    torch.cuda.set_device(local)
    from simplenavierstokessolver_gb300 import Case, kernel_launches
    from simplenavierstokessolver_gb300 import _native as N

    lib = N.lib()
    if args.large_only or args.serving_only:
        # one leg alone, for its own measurement runs (not a bench line)
        part = large_instance(args, torch, steps=args.large_steps, acc_steps=args.large_acc_steps) \
            if args.large_only else serving(args)
        if rank == 0:
            print(json.dumps({"leg": "large_instance" if args.large_only else "serving", **part}))
        return 0
    case = Case(args.nx, args.ny, ly=2.0, Ra=args.Ra, Pr=args.Pr)
    # the headline's arithmetic form: the parallel form (within 1e-12 of the
    # oracle after the stated step counts) where the grid supports it
    form = args.form
    if form == "parallel":
        try:
            case.set_form(True)
        except N.SnsError:
            form = "exact"
    stream = torch.cuda.ExternalStream(case.stream())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    cells = args.nx * args.ny

    def flush_l2():
        with torch.cuda.stream(stream):
            flush.zero_()

    clocks = ClockSampler(local)
    clocks.start()
    for _ in range(args.warmup):
        case.run(1)
        flush_l2()
    torch.cuda.synchronize()

    # ---- pass A: headline, uninstrumented
    barrier(world)
    torch.cuda.synchronize()
    t_region = time.perf_counter()
    launches0 = kernel_launches()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for a, b in ev:
        a.record(stream)
        case.run(1)
        b.record(stream)
        flush_l2()
    torch.cuda.synchronize()
    clocks.mark(t_region, time.perf_counter())
    barrier(world)
    launches = kernel_launches() - launches0
    ms = sum(a.elapsed_time(b) for a, b in ev)
    ms = max_over_ranks(ms, world)
    value = cells * args.steps * world / (ms * 1e-3)

    # ---- pass B: per-kernel device times (events around each launch)
    lib.sns_profile(case.fluid, 1)
    for _ in range(args.steps):
        case.run(1)
        flush_l2()
    kinds = 16
    kms = (N.c_double * kinds)()
    kcnt = (N.c_longlong * kinds)()
    nk = lib.sns_profile_read(case.fluid, kms, kcnt, kinds)
    lib.sns_profile(case.fluid, 0)
    clk = clocks.stop()
    kernels = {}
    total_k = sum(kms[k] for k in range(nk))
    for k in range(nk):
        if kcnt[k]:
            name = lib.sns_profile_kind_name(k).decode()
            kernels[name] = {"launches": int(kcnt[k]), "ms": kms[k], "avg_us": 1e3 * kms[k] / kcnt[k],
                             "share": kms[k] / total_k if total_k else None}
    dom = max(kernels, key=lambda n: kernels[n]["ms"])
    peak, peak_kind = load_peaks()
    # the FP64 issue rate of this GPU, measured in this run (independent FP64
    # additions and multiplications on every SM: sns_fp64_issue_rate)
    rate = N.fp64_issue_rate()
    fp64_peak = 0.5 * (rate["dadd_gops"] + rate["dmul_gops"])
    fp64_source = (f"measured in this run by sns_fp64_issue_rate: DADD {rate['dadd_gops']:.1f}, "
                   f"DMUL {rate['dmul_gops']:.1f} Gop/s")
    vel_model = "velocity_update_p2" if power_of_two_grid(case.grid()) else "velocity_update"
    bpc, opc = KERNEL_MODEL.get(vel_model if dom == "velocity_update" else dom, (None, None))
    if dom == "poisson_forward_fft":
        opc = fft_ops_per_cell(args.ny, True)
    if dom == "poisson_inverse_fft":
        opc = fft_ops_per_cell(args.ny, False)
    if dom == "poisson_fused":
        opc = fft_ops_per_cell(args.ny, True) + fft_ops_per_cell(args.ny, False) + 5.0 + 27.0
    measured_ops = form == "parallel" and (args.nx, args.ny) == (512, 1024) and dom in PARALLEL_FP64_OPS
    if measured_ops:
        opc = PARALLEL_FP64_OPS[dom]
    avg_s = kernels[dom]["avg_us"] * 1e-6
    achieved = bpc * cells / avg_s / 1e9 if bpc else None
    roofline = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak if achieved else None,
                "traffic": PROFILED_TRAFFIC.get((dom, args.nx, args.ny)),
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback",
                "algorithmic_bytes_per_launch": bpc * cells if bpc else None,
                "note": "FP64-pipe bound on GB300: see fp64_roofline"}
    fp64 = None
    if opc:
        ach = opc * cells / avg_s / 1e9
        fp64 = {"kernel": dom, "achieved": ach, "peak": fp64_peak, "unit": "Gop/s (FP64 instructions)",
                "frac": ach / fp64_peak, "ops_per_cell": opc, "peak_source": fp64_source,
                "ops_source": ("ncu instruction counts of the parallel form's kernel at 512x1024 "
                               "(profiles/plain_parallel_fp64_counts_512x1024.md)") if measured_ops
                else "counted from the exact form's kernels"}
    # the whole explicit step against the FP64 issue rate: FP64 operations per
    # cell-step from the kernels' counts (3 substages of temperature, velocity,
    # forward DFT, sweep, inverse DFT and correction)
    # (counted for the exact form; the parallel form's contracted kernels
    # issue fewer FP64 instructions than these counts)
    ops_step = 3 * (KERNEL_MODEL["temperature_update"][1] + KERNEL_MODEL[vel_model][1] +
                    fft_ops_per_cell(args.ny, True) + KERNEL_MODEL["poisson_tridiagonal"][1] +
                    fft_ops_per_cell(args.ny, False) + KERNEL_MODEL["correct_and_pressure"][1])
    if form == "parallel" and (args.nx, args.ny) == (512, 1024):
        ops_step = 3 * sum(PARALLEL_FP64_OPS.values())
    step_fp64 = {"form": form, "ops_per_cell_step": ops_step, "achieved": value * ops_step / 1e9, "peak": fp64_peak,
                 "unit": "Gop/s (FP64 instructions)", "frac": value * ops_step / 1e9 / fp64_peak,
                 "peak_source": fp64_source}

    # ---- the same workload in the other arithmetic form, same protocol
    other_form = "exact" if form == "parallel" else "parallel"
    other = None
    with Case(args.nx, args.ny, ly=2.0, Ra=args.Ra, Pr=args.Pr) as pc:
        try:
            pc.set_form(other_form == "parallel")
        except N.SnsError as err:
            other = {"unavailable": str(err)}
        if other is None:
            pstream = torch.cuda.ExternalStream(pc.stream())
            for _ in range(args.warmup):
                pc.run(1)
                with torch.cuda.stream(pstream):
                    flush.zero_()
            torch.cuda.synchronize()
            pev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                   for _ in range(args.steps)]
            for a, b in pev:
                a.record(pstream)
                pc.run(1)
                b.record(pstream)
                with torch.cuda.stream(pstream):
                    flush.zero_()
            torch.cuda.synchronize()
            pms = max_over_ranks(sum(a.elapsed_time(b) for a, b in pev), world)
            lib.sns_profile(pc.fluid, 1)
            for _ in range(args.steps):
                pc.run(1)
                with torch.cuda.stream(pstream):
                    flush.zero_()
            pkms = (N.c_double * kinds)()
            pkcnt = (N.c_longlong * kinds)()
            pnk = lib.sns_profile_read(pc.fluid, pkms, pkcnt, kinds)
            lib.sns_profile(pc.fluid, 0)
            ptot = sum(pkms[k] for k in range(pnk))
            pkern = {lib.sns_profile_kind_name(k).decode(): {"launches": int(pkcnt[k]),
                                                             "avg_us": 1e3 * pkms[k] / pkcnt[k],
                                                             "share": pkms[k] / ptot if ptot else None}
                     for k in range(pnk) if pkcnt[k]}
            other = {"form": other_form, "value": cells * args.steps * world / (pms * 1e-3), "unit": "cell-steps/s",
                     "ms_per_step": pms / args.steps, "headline_speedup_over_this": pms / ms, "kernels": pkern}
    forms = {"headline": form, "other": other,
             "exact": "every operation of the reference in its order, Thomas recurrence: identical to the oracle "
                      "bit for bit (tests/test_gpu_long_parity.py)",
             "parallel": "Poisson lines by the partition method + warp-shuffle PCR, FMA-contracted kernels: within "
                         "1e-12 relative L2 of the oracle per field after 1000 / 2000 steps "
                         "(tests/test_gpu_parallel_form.py)"}

    # ---- end to end through the C ABI with host buffers
    # each step: host arrays -> device, one time step (param_decide_dt + the 3
    # substages), device -> host arrays. Headline: ux, uy, p and temp, the
    # whole input and output of a step (sns_sync_state_to_device / _to_host),
    # around sns_run(1), the fused form of the reference's main-loop step.
    # Beside it the same step with every host array of the structures
    # (sns_sync_to_device / _to_host), and the step issued as the
    # reference-named calls (param_decide_dt, temperature_*, fluid_*).
    e2e_steps = max(2, min(args.steps, 10))
    host = case.host_arrays()
    case.sync_to_host()
    state_bytes = sum(host[k].size * 8 for k in ("ux", "uy", "p", "temp"))
    h2d_full = sum(host[k].size * 8 for k in ("ux", "uy", "p", "psi", "temp", "srcuxa", "srcuya", "srctempa"))
    d2h_full = h2d_full + host["tempforcex"].size * 8

    breakdown = {}

    def e2e_rate(step, state_only):
        up = case.sync_state_to_device if state_only else case.sync_to_device
        down = case.sync_state_to_host if state_only else case.sync_to_host
        torch.cuda.synchronize()
        barrier(world)
        t = [0.0, 0.0, 0.0]
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            a = time.perf_counter()
            up()
            b = time.perf_counter()
            step()
            c = time.perf_counter()
            down()
            d = time.perf_counter()
            t[0] += b - a
            t[1] += c - b
            t[2] += d - c
        total = time.perf_counter() - t0
        breakdown[(state_only, step)] = {"to_device_ms": 1e3 * t[0] / e2e_steps, "step_ms": 1e3 * t[1] / e2e_steps,
                                         "to_host_ms": 1e3 * t[2] / e2e_steps}
        return cells * e2e_steps * world / max_over_ranks(total, world)

    run1 = lambda: case.run(1)  # noqa: E731
    e2e_full = e2e_rate(run1, False)
    e2e_calls = e2e_rate(lambda: case.run_calls(1), False)
    e2e_value = e2e_rate(run1, True)
    e2e = {"value": e2e_value, "unit": "cell-steps/s", "h2d_bytes_per_step": state_bytes,
           "d2h_bytes_per_step": state_bytes, "steps": e2e_steps,
           "breakdown_host_wall": breakdown[(True, run1)],
           "link_gbs": {"to_device": state_bytes / (breakdown[(True, run1)]["to_device_ms"] * 1e-3) / 1e9,
                        "to_host": state_bytes / (breakdown[(True, run1)]["to_host_ms"] * 1e-3) / 1e9},
           "path": "sns_sync_state_to_device + sns_run(1) (param_decide_dt + 3 fused substages) "
                   "+ sns_sync_state_to_host",
           "all_host_arrays": {"value": e2e_full, "unit": "cell-steps/s", "h2d_bytes_per_step": h2d_full,
                               "d2h_bytes_per_step": d2h_full,
                               "path": "sns_sync_to_device + sns_run(1) + sns_sync_to_host"},
           "reference_named_calls": {"value": e2e_calls, "unit": "cell-steps/s", "h2d_bytes_per_step": h2d_full,
                                     "d2h_bytes_per_step": d2h_full,
                                     "path": "sns_sync_to_device + param_decide_dt + temperature_*/fluid_* calls "
                                             "+ sns_sync_to_host"}}
    case.close()

    extra = {}
    if not args.plain_only:
        extra["fp32_stencil"] = fp32_single(args, torch)
        extra["fp32_stencil"]["vs_plain_fp64"] = extra["fp32_stencil"]["value"] / value
        extra["fp32_stencil"]["accuracy_vs_fp64"] = fp32_accuracy(args)
        extra["ensemble_64"] = ensemble_throughput(args, torch)
        if args.ens_acc_steps > 0:
            extra["ensemble_64"]["accuracy_vs_fp64"] = ensemble_accuracy(args)
        # the same case and ensemble with float-float stencil terms and increments
        comp = fp32_single(args, torch, compensated=True)
        comp["vs_plain_fp64"] = comp["value"] / value
        comp["accuracy_vs_fp64"] = fp32_accuracy(args, compensated=True)
        ens = ensemble_throughput(args, torch, compensated=True)
        ens["ratio_vs_plain_concurrent"] = ens["batched_compensated"] / extra["ensemble_64"][
            "plain_fp64_concurrent_streams"]
        ens["ratio_vs_plain_one_by_one"] = ens["batched_compensated"] / extra["ensemble_64"]["plain_fp64_one_by_one"]
        if args.ens_acc_steps > 0:
            ens["accuracy_vs_fp64"] = ensemble_accuracy(args, compensated=True)
        comp["ensemble_64"] = ens
        extra["fp32_compensated"] = comp
        extra["serving"] = serving(args)
        if args.large_steps > 0:
            extra["large_instance"] = large_instance(args, torch, steps=args.large_steps,
                                                     acc_steps=args.large_acc_steps)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        from oracle.build import build as build_oracle
        from oracle.bindings import Config

        build_oracle()
        threads = os.cpu_count() or 1
        rate, n, el = cpu_oracle_rate(Config(args.nx, args.ny, ly=2.0, Ra=args.Ra, Pr=args.Pr), args.cpu_seconds,
                                      threads)
        cpu = {"value": rate, "unit": "cell-steps/s", "cores": threads, "kind": "port",
               "sample": f"{n} time steps of {args.nx}x{args.ny} in {el:.1f} s on {threads} threads "
                         "(CPU oracle, bit-identical to the reference)"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "cell-steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (reference initial condition, srand(0))", "config": dict(workload_config(args), form=form),
            "roofline": roofline, "fp64_roofline": fp64, "step_fp64_roofline": step_fp64, "kernels": kernels,
            "forms": forms, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": int(launches), "clocks": clk,
        }
        line.update(extra)
        print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--nx", type=int, default=512)
    ap.add_argument("--ny", type=int, default=1024)
    ap.add_argument("--Ra", type=float, default=1e9)
    ap.add_argument("--Pr", type=float, default=1.0)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--plain-only", action="store_true", help="skip the FP32-stencil, ensemble and serving parts")
    ap.add_argument("--large-only", action="store_true", help="run the 2048x4096 leg alone")
    ap.add_argument("--serving-only", action="store_true", help="run the serving leg alone")
    ap.add_argument("--form", default="parallel", choices=["parallel", "exact"],
                    help="arithmetic form of the headline plain FP64 step (sns_set_form)")
    ap.add_argument("--acc-steps", type=int, default=2000, help="steps of the FP32-vs-FP64 accuracy run")
    ap.add_argument("--ens-steps", type=int, default=50)
    ap.add_argument("--ens-acc-steps", type=int, default=500, help="steps of the ensemble FP32-vs-FP64 accuracy run")
    ap.add_argument("--large-steps", type=int, default=500, help="timed steps of the 2048x4096 Ra=1e10 instance")
    ap.add_argument("--large-acc-steps", type=int, default=200,
                    help="steps of the batched forms' accuracy run at 2048x4096 (0: skip)")
    ap.add_argument("--serve-rate", type=float, default=6.0)
    ap.add_argument("--serve-seconds", type=float, default=12.0)
    ap.add_argument("--serve-hbm", type=int, default=2048, help="serving arena in MiB")
    ap.add_argument("--serve-chunk", type=int, default=10)
    ap.add_argument("--serve-compensated", type=int, default=1,
                    help="requests in the compensated (float-float) form (1) or FP32 (0)")
    ap.add_argument("--serve-acc-sample", type=int, default=3,
                    help="served requests checked against the FP64 path (the cheapest ones)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_setup()
    if args.impl == "reference":
        return reference_arm(args, world, rank)
    return gpu_arm(args, world, rank, local)


if __name__ == "__main__":
    sys.exit(main())
