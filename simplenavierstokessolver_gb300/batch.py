"""Python mirror of the batched FP32-stencil / FP64-Poisson engine
(include/sns_batch.h): many independent Rayleigh-Benard cases advanced by the
same launches, fields device-resident, admission by HBM footprint."""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_double, c_int, c_longlong
from dataclasses import dataclass

import numpy as np

from . import _native as N


CaseDesc = N.CaseDesc
_PD = POINTER(c_double)


def _lib():
    return N.lib()


@dataclass
class Desc:
    itot: int
    jtot: int
    ly: float = 2.0
    stretch: float = 1e9
    Ra: float = 1e8
    Pr: float = 1.0
    with_temperature: bool = True
    with_thermal_forcing: bool = True
    steps: int = 0
    seed: int = 0
    fixed_dt: float = 0.0
    # float-float stencil terms and increments (about 48 bits) instead of FP32
    compensated: bool = False

    def c(self) -> CaseDesc:
        return CaseDesc(self.itot, self.jtot, self.ly, self.stretch, self.Ra, self.Pr, int(self.with_temperature),
                        int(self.with_thermal_forcing), int(self.steps), int(self.seed), float(self.fixed_dt),
                        int(self.compensated))


def _ptr(a):
    return a.ctypes.data_as(_PD) if a is not None else None


def case_bytes(desc: Desc) -> int:
    d = desc.c()
    return int(_lib().sns_batch_case_bytes(ctypes.byref(d)))


def initial_temperature(desc: Desc) -> np.ndarray:
    t = np.zeros((desc.jtot + 2, desc.itot + 2))
    d = desc.c()
    N.check(_lib().sns_batch_initial_temperature(ctypes.byref(d), _ptr(t)), "sns_batch_initial_temperature")
    return t


class Batch:
    def __init__(self, hbm_bytes: int, max_cases: int = 256):
        self.lib = _lib()
        self.h = self.lib.sns_batch_create(hbm_bytes, max_cases)
        if not self.h:
            raise N.SnsError(N.SNS_ERR_OOM, "sns_batch_create")
        self.descs = {}

    def close(self):
        if getattr(self, "h", None):
            self.lib.sns_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def free_bytes(self) -> int:
        return int(self.lib.sns_batch_free_bytes(self.h))

    def add(self, desc: Desc, temp_init: np.ndarray | None = None) -> int:
        d = desc.c()
        slot = c_int(-1)
        t = None if temp_init is None else np.ascontiguousarray(temp_init, dtype=np.float64)
        N.check(self.lib.sns_batch_add(self.h, ctypes.byref(d), _ptr(t), ctypes.byref(slot)), "sns_batch_add")
        self.descs[slot.value] = desc
        return slot.value

    def add_restart(self, desc: Desc, dirname: str) -> int:
        """admit a case from a directory in the reference's save layout"""
        d = desc.c()
        slot = c_int(-1)
        N.check(self.lib.sns_batch_add_restart(self.h, ctypes.byref(d), dirname.encode(), ctypes.byref(slot)),
                "sns_batch_add_restart")
        self.descs[slot.value] = desc
        return slot.value

    def checkpoint(self, slot: int, dirname: str):
        """the case's state in the reference's save layout"""
        N.check(self.lib.sns_batch_checkpoint(self.h, slot, dirname.encode()), "sns_batch_checkpoint")

    def try_add(self, desc: Desc) -> int | None:
        d = desc.c()
        slot = c_int(-1)
        rc = self.lib.sns_batch_add(self.h, ctypes.byref(d), None, ctypes.byref(slot))
        if rc == N.SNS_ERR_OOM:
            return None
        N.check(rc, "sns_batch_add")
        self.descs[slot.value] = desc
        return slot.value

    def remove(self, slot: int):
        N.check(self.lib.sns_batch_remove(self.h, slot), "sns_batch_remove")
        self.descs.pop(slot, None)

    def step(self, n: int = 1):
        N.check(self.lib.sns_batch_step(self.h, n), "sns_batch_step")

    def synchronize(self):
        N.check(self.lib.sns_batch_synchronize(self.h), "sns_batch_synchronize")

    def stream(self) -> int:
        return self.lib.sns_batch_stream(self.h) or 0

    def active_cells(self) -> int:
        return int(self.lib.sns_batch_active_cells(self.h))

    def status(self, slot: int):
        """time, next dt, step, done; finite is False once the case wrote a
        NaN or infinity (sns_batch_case_status returns SNS_ERR_NONFINITE)"""
        return status_of(self.h, slot)

    def set_persistent(self, on: bool):
        """one persistent cooperative launch per substage (the same arithmetic)"""
        N.check(self.lib.sns_batch_set_persistent(self.h, int(on)), "sns_batch_set_persistent")

    def set_wait_limit(self, polls: int, stale: bool = False):
        N.check(self.lib.sns_batch_set_wait_limit(self.h, polls, int(stale)), "sns_batch_set_wait_limit")

    def tuning(self) -> dict:
        t = N.Tuning()
        N.check(self.lib.sns_batch_get_tuning(self.h, ctypes.byref(t)), "sns_batch_get_tuning")
        return {f: getattr(t, f) for f, _ in N.Tuning._fields_}

    def set_tuning(self, **kw):
        t = N.Tuning(**{**self.tuning(), **kw})
        N.check(self.lib.sns_batch_set_tuning(self.h, ctypes.byref(t)), "sns_batch_set_tuning")

    def autotune(self, steps: int = 5):
        """pick launch shapes by timing candidates on the resident cases
        (their state is left unchanged); returns the shapes and ms per step"""
        t, ms = N.Tuning(), ctypes.c_double()
        N.check(self.lib.sns_batch_autotune(self.h, steps, ctypes.byref(t), ctypes.byref(ms)), "sns_batch_autotune")
        return {f: getattr(t, f) for f, _ in N.Tuning._fields_}, ms.value

    def diagnostics(self, slot: int) -> np.ndarray:
        return diagnostics_of(self.h, slot)

    def state(self, slot: int):
        d = self.descs[slot]
        su, sc = (d.jtot + 2, d.itot + 1), (d.jtot + 2, d.itot + 2)
        out = {"ux": np.zeros(su), "uy": np.zeros(sc), "p": np.zeros(sc), "psi": np.zeros(sc), "temp": np.zeros(sc)}
        N.check(self.lib.sns_batch_state(self.h, slot, _ptr(out["ux"]), _ptr(out["uy"]), _ptr(out["p"]),
                                         _ptr(out["psi"]), _ptr(out["temp"])), "sns_batch_state")
        return out


def status_of(batch_handle, slot: int) -> dict:
    t, dt, st, done = c_double(), c_double(), c_longlong(), c_int()
    rc = _lib().sns_batch_case_status(batch_handle, slot, ctypes.byref(t), ctypes.byref(dt), ctypes.byref(st),
                                      ctypes.byref(done))
    if rc != N.SNS_ERR_NONFINITE:
        N.check(rc, "sns_batch_case_status")
    return {"time": t.value, "dt": dt.value, "step": st.value, "done": bool(done.value),
            "finite": rc != N.SNS_ERR_NONFINITE}


def diagnostics_of(batch_handle, slot: int) -> np.ndarray:
    out = np.zeros(11)
    N.check(_lib().sns_batch_diagnostics(batch_handle, slot, _ptr(out)), "sns_batch_diagnostics")
    return out


def state_of(batch_handle, slot: int, desc: Desc):
    su, sc = (desc.jtot + 2, desc.itot + 1), (desc.jtot + 2, desc.itot + 2)
    out = {"ux": np.zeros(su), "uy": np.zeros(sc), "p": np.zeros(sc), "psi": np.zeros(sc), "temp": np.zeros(sc)}
    N.check(_lib().sns_batch_state(batch_handle, slot, _ptr(out["ux"]), _ptr(out["uy"]), _ptr(out["p"]),
                                   _ptr(out["psi"]), _ptr(out["temp"])), "sns_batch_state")
    return out


def serve(descs: list[Desc], arrivals: list[float], hbm_bytes: int, max_cases: int = 256, chunk_steps: int = 10,
          keep_states: bool = False):
    """Runs sns_serve (continuous batching in real time). Returns admission
    and completion times (seconds from the start), the busy span, whether
    each request's final state is finite (no NaN or infinity written) and,
    with keep_states, each request's final fields read just before
    retirement."""
    n = len(descs)
    arr = (N.CaseDesc * n)(*[d.c() for d in descs])
    at = np.ascontiguousarray(arrivals, dtype=np.float64)
    admit, done = np.zeros(n), np.zeros(n)
    finite = np.ones(n, dtype=bool)
    busy = c_double()
    states = {}

    def on_done(req, bh, slot, user):
        finite[req] = status_of(bh, slot)["finite"]
        if keep_states:
            states[req] = state_of(bh, slot, descs[req])

    cb = N.DONE_FN(on_done)
    rc = _lib().sns_serve(arr, _ptr(at), n, hbm_bytes, max_cases, chunk_steps, _ptr(admit), _ptr(done),
                          ctypes.byref(busy), ctypes.cast(cb, ctypes.c_void_p), None)
    N.check(rc, "sns_serve")
    return {"admit": admit, "done": done, "busy_s": busy.value, "finite": finite, "states": states}
