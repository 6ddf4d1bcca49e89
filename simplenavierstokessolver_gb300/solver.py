"""Host-side mirror of the reference's operator interface, over the C ABI.

``Case`` owns one param_t / parallel_t / fluid_t / temperature_t quartet
created by libsns_gpu.so and exposes the reference's hot-path calls under
their own names (``fluid_update_velocity``, ``fluid_compute_potential``, ...),
the substage sequence of the reference's ``integrate()`` (src/main.c:79-101)
and the step loop of its ``main()`` (src/main.c:28-35). Fields are exchanged
as numpy arrays in the reference's layouts (include/arrays/*.h): shape
(jtot+2, itot+1) for ux and (jtot+2, itot+2) for uy, p, psi and temp, halo
rows and wall columns included.

Every method raises ``SnsError`` with the library's message on a nonzero
status; nothing here computes physics on the CPU.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N


def _view(ptr, shape):
    n = int(np.prod(shape))
    return np.ctypeslib.as_array(ptr, shape=(n,)).reshape(shape)


class Case:
    def __init__(self, itot: int, jtot: int, ly: float = 2.0, stretch: float = 1e9, Ra: float = 1e8,
                 Pr: float = 1.0, with_temperature: bool = True, with_thermal_forcing: bool = True,
                 costs=(1.0, 2.0, 2.0, 3.0)):
        self.lib = N.lib()
        self.itot, self.jtot = itot, jtot
        self.param = self.lib.sns_param_create(itot, jtot, ly, stretch, Ra, Pr, int(with_temperature),
                                               int(with_thermal_forcing))
        if not self.param:
            raise N.SnsError(N.SNS_ERR_ARG, "sns_param_create")
        self.set_costs(costs)
        # srand(0) as the reference's parallel_init does on rank 0, before temperature_init
        self.parallel = self.lib.sns_parallel_create()
        self.fluid = self.lib.fluid_init(self.param, self.parallel)
        if not self.fluid:
            msg = N.last_error()
            self._free_param()
            raise N.SnsError(N.SNS_ERR_UNSUPPORTED, f"fluid_init ({msg})")
        self.temperature = self.lib.temperature_init(self.param, self.parallel)
        if not self.temperature:
            msg = N.last_error()
            self.close()
            raise N.SnsError(N.SNS_ERR_UNSUPPORTED, f"temperature_init ({msg})")

    # ------------------------------------------------------------ lifecycle
    def _free_param(self):
        if getattr(self, "parallel", None):
            self.lib.sns_parallel_destroy(self.parallel)
            self.parallel = None
        if getattr(self, "param", None):
            self.lib.sns_param_destroy(self.param)
            self.param = None

    def close(self):
        if getattr(self, "temperature", None):
            self.lib.temperature_finalise(self.temperature)
            self.temperature = None
        if getattr(self, "fluid", None):
            self.lib.fluid_finalise(self.fluid)
            self.fluid = None
        self._free_param()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------ parameters
    @property
    def p(self) -> N.Param:
        return self.param.contents

    def set_costs(self, w):
        for y in range(2):
            for x in range(2):
                self.p.expimp_wtimes[y][x] = float(w[2 * y + x])

    def set_dt(self, dt: float, implicitx: int = 0, implicity: int = 0):
        self.p.dt = dt
        self.p.implicitx = implicitx
        self.p.implicity = implicity

    def get_dt(self):
        p = self.p
        return {"dt": p.dt, "implicitx": p.implicitx, "implicity": p.implicity, "time": p.time, "step": p.step}

    def set_time(self, time: float, step: int):
        self.p.time = time
        self.p.step = step

    def grid(self):
        p, n = self.p, self.itot
        return {"xf": np.ctypeslib.as_array(p.xf, (n + 1,)).copy(), "xc": np.ctypeslib.as_array(p.xc, (n + 2,)).copy(),
                "dxf": np.ctypeslib.as_array(p.dxf, (n,)).copy(), "dxc": np.ctypeslib.as_array(p.dxc, (n + 1,)).copy(),
                "dy": p.dy}

    # ---------------------------------------------------------------- state
    def shapes(self):
        return (self.jtot + 2, self.itot + 1), (self.jtot + 2, self.itot + 2)

    def host_arrays(self):
        """numpy views of the structures' host arrays (valid after sync_to_host)."""
        su, sc = self.shapes()
        f, t = self.fluid.contents, self.temperature.contents
        return {"ux": _view(f.ux, su), "uy": _view(f.uy, sc), "p": _view(f.p, sc), "psi": _view(f.psi, sc),
                "temp": _view(t.temp, sc),
                "srcuxa": _view(f.srcuxa, (self.jtot, self.itot - 1)),
                "srcuya": _view(f.srcuya, (self.jtot, self.itot)),
                "srctempa": _view(t.srctempa, (self.jtot, self.itot)),
                "tempforcex": _view(t.tempforcex, (self.jtot, self.itot - 1))}

    def sync_to_host(self):
        N.check(self.lib.sns_sync_to_host(self.param, self.fluid, self.temperature), "sns_sync_to_host")

    def sync_to_device(self):
        N.check(self.lib.sns_sync_to_device(self.param, self.fluid, self.temperature), "sns_sync_to_device")

    def sync_state_to_host(self):
        """ux, uy, p and temp alone (the whole-step state)"""
        N.check(self.lib.sns_sync_state_to_host(self.param, self.fluid, self.temperature), "sns_sync_state_to_host")

    def sync_state_to_device(self):
        N.check(self.lib.sns_sync_state_to_device(self.param, self.fluid, self.temperature),
                "sns_sync_state_to_device")

    def get_state(self):
        self.sync_to_host()
        h = self.host_arrays()
        return {k: h[k].copy() for k in ("ux", "uy", "p", "psi", "temp")}

    def get_sources(self):
        self.sync_to_host()
        h = self.host_arrays()
        return {k: h[k].copy() for k in ("srcuxa", "srcuya", "srctempa")}

    def set_state(self, ux, uy, p, temp, sources=None):
        h = self.host_arrays()
        h["ux"][...] = ux
        h["uy"][...] = uy
        h["p"][...] = p
        h["temp"][...] = temp
        if sources is not None:
            for k, v in sources.items():
                h[k][...] = v
        self.sync_to_device()

    # ---------------------------------------------- reference hot-path calls
    def fluid_update_velocity(self, rk):
        N.check(self.lib.fluid_update_velocity(self.param, self.parallel, rk, self.fluid, self.temperature),
                "fluid_update_velocity")

    def fluid_compute_potential(self, rk):
        N.check(self.lib.fluid_compute_potential(self.param, self.parallel, rk, self.fluid), "fluid_compute_potential")

    def fluid_correct_velocity(self, rk):
        N.check(self.lib.fluid_correct_velocity(self.param, self.parallel, rk, self.fluid), "fluid_correct_velocity")

    def fluid_update_pressure(self, rk):
        N.check(self.lib.fluid_update_pressure(self.param, self.parallel, rk, self.fluid), "fluid_update_pressure")

    def temperature_compute_force(self):
        N.check(self.lib.temperature_compute_force(self.param, self.parallel, self.temperature),
                "temperature_compute_force")

    def temperature_update_temp(self, rk):
        N.check(self.lib.temperature_update_temp(self.param, self.parallel, rk, self.fluid, self.temperature),
                "temperature_update_temp")

    def update_boundaries(self):
        """the four boundary calls at the top of a substage (src/main.c:82-87) on the host arrays"""
        f, t = self.fluid.contents, self.temperature.contents
        N.check(self.lib.fluid_update_boundaries_ux(self.param, self.parallel, f.ux), "fluid_update_boundaries_ux")
        N.check(self.lib.fluid_update_boundaries_uy(self.param, self.parallel, f.uy), "fluid_update_boundaries_uy")
        N.check(self.lib.fluid_update_boundaries_p(self.param, self.parallel, f.p), "fluid_update_boundaries_p")
        if self.p.with_temperature:
            N.check(self.lib.temperature_update_boundaries_temp(self.param, self.parallel, t.temp),
                    "temperature_update_boundaries_temp")

    def estimate_cost(self):
        """param_estimate_cost: the deterministic model fills expimp_wtimes"""
        N.check(self.lib.param_estimate_cost(self.param, self.parallel), "param_estimate_cost")
        p = self.p
        return [p.expimp_wtimes[y][x] for y in range(2) for x in range(2)]

    def measure_cost(self, reps: int = 20):
        """seconds per substage of EXP/IMP combinations, CUDA-event timed
        (index 2*implicity + implicitx)"""
        out = (ctypes.c_double * 4)()
        N.check(self.lib.sns_measure_cost(self.param, self.parallel, reps, out), "sns_measure_cost")
        return list(out)

    def param_decide_dt(self):
        N.check(self.lib.param_decide_dt(self.param, self.parallel, self.fluid), "param_decide_dt")

    def substage(self, rk):
        """one RK substage as the reference's integrate() issues it, call by call"""
        self.update_boundaries()
        if self.p.with_temperature:
            self.temperature_compute_force()
            self.temperature_update_temp(rk)
        self.fluid_update_velocity(rk)
        self.fluid_compute_potential(rk)
        self.fluid_correct_velocity(rk)
        self.fluid_update_pressure(rk)

    def run_calls(self, nsteps: int, decide: bool = True):
        """main-loop steps issued through the individual reference-named calls"""
        for _ in range(nsteps):
            if decide:
                self.param_decide_dt()
            for rk in range(3):
                self.substage(rk)
            self.p.step += 1
            self.p.time += self.p.dt
        self.synchronize()

    def diagnostics(self) -> np.ndarray:
        """the reference's 11 log quantities from the device state (sns_diagnostics)"""
        out = np.zeros(11)
        N.check(self.lib.sns_diagnostics(self.param, self.fluid, self.temperature,
                                         out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))), "sns_diagnostics")
        return out

    # ------------------------------------------------------ checkpoints
    def checkpoint(self, dirname: str):
        """asynchronous: the files appear after checkpoint_wait()"""
        N.check(self.lib.sns_checkpoint(self.param, self.fluid, self.temperature, dirname.encode()), "sns_checkpoint")

    def checkpoint_wait(self):
        N.check(self.lib.sns_checkpoint_wait(self.fluid), "sns_checkpoint_wait")

    def restart(self, dirname: str):
        N.check(self.lib.sns_restart(self.param, self.fluid, self.temperature, dirname.encode()), "sns_restart")

    # ------------------------------------------------------- fused fast path
    def integrate(self):
        N.check(self.lib.sns_integrate(self.param, self.parallel, self.fluid, self.temperature), "sns_integrate")

    def run(self, nsteps: int):
        N.check(self.lib.sns_run(self.param, self.parallel, self.fluid, self.temperature, nsteps), "sns_run")

    def set_form(self, parallel: bool):
        """the arithmetic form of the plain path: the reference's operations
        and order (identical results, the default) or the parallel form
        (Poisson lines by the partition method with parallel cyclic
        reduction, fused multiply-adds; within 1e-12 relative L2)"""
        N.check(self.lib.sns_set_form(self.fluid, N.SNS_FORM_PARALLEL if parallel else N.SNS_FORM_EXACT),
                "sns_set_form")

    def set_wait_limit(self, polls: int, stale: bool = False):
        N.check(self.lib.sns_set_wait_limit(self.fluid, polls, int(stale)), "sns_set_wait_limit")

    def set_fused(self, on: bool):
        """one cooperative launch per Poisson solve (default) or three kernels"""
        N.check(self.lib.sns_set_fused(self.fluid, int(on)), "sns_set_fused")

    def synchronize(self):
        N.check(self.lib.sns_synchronize(self.fluid), "sns_synchronize")

    def stream(self) -> int:
        return self.lib.sns_stream(self.fluid) or 0


def kernel_launches() -> int:
    return int(N.lib().sns_kernel_launches())


def save_dirname(step: int, root: str = "output/save") -> str:
    """the directory the reference's save() uses for a step (src/save.c:40-50)"""
    return f"{root}/step{step:010d}"


def npy_write(path: str, array: np.ndarray):
    """an NPY file in the reference's format (float64 or int32, C order)"""
    a = np.asarray(array, order="C")
    dtype = {np.dtype(np.float64): b"'float64'", np.dtype(np.int32): b"'int32'"}[a.dtype]
    shape = (ctypes.c_size_t * max(a.ndim, 1))(*a.shape)
    N.check(N.lib().sns_npy_write(path.encode(), dtype, a.ndim, shape, a.ctypes.data, a.nbytes), "sns_npy_write")


def npy_read(path: str, shape, dtype=np.float64) -> np.ndarray:
    a = np.empty(shape, dtype=dtype)
    d = {np.dtype(np.float64): b"'float64'", np.dtype(np.int32): b"'int32'"}[a.dtype]
    s = (ctypes.c_size_t * max(a.ndim, 1))(*a.shape)
    N.check(N.lib().sns_npy_read(path.encode(), d, a.ndim, s, a.ctypes.data, a.nbytes), "sns_npy_read")
    return a


class Statistics:
    """statistics_t of the reference (include/statistics.h) over a Case:
    running sums of u and u^2 on the device (statistics_collect), written as
    the reference's statistics_output files."""

    def __init__(self, case: Case):
        self.case = case
        self.lib = case.lib
        self.s = self.lib.statistics_init(case.param, case.parallel)
        if not self.s:
            raise N.SnsError(N.SNS_ERR_ARG, "statistics_init")

    def collect(self):
        c = self.case
        N.check(self.lib.statistics_collect(c.param, c.parallel, c.fluid, c.temperature, self.s),
                "statistics_collect")

    @property
    def num(self) -> int:
        return self.s.contents.num

    def output_to(self, dirname: str):
        N.check(self.lib.sns_statistics_output_to(self.case.param, self.s, dirname.encode()),
                "sns_statistics_output_to")

    def close(self):
        if getattr(self, "s", None):
            self.lib.statistics_finalise(self.s)
            self.s = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def cost_model(itot: int, jtot: int, sm_count: int = 152, clock_ghz: float = 2.07, with_temperature: bool = True):
    """predicted seconds per substage, index 2*implicity + implicitx (host only)"""
    out = (ctypes.c_double * 4)()
    N.check(N.lib().sns_cost_model(itot, jtot, sm_count, clock_ghz, int(with_temperature), out), "sns_cost_model")
    return list(out)
