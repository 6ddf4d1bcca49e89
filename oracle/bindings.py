"""TEST INFRASTRUCTURE ONLY -- ctypes bindings for the CPU oracle.

Two libraries are bound here:

* ``build/liboracle.so``  -- the C restatement of the reference's FP64 step
  (``sns_oracle.c``), built on every machine by ``oracle/build.py``;
* ``_ref/libsnsref.so``   -- the reference's own sources compiled with the
  single-rank MPI / FFTW stand-ins (``shim/``), built only where the reference
  source tree is mounted.

Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module. Arrays follow the reference layouts
(include/arrays/*.h): numpy shape (jtot+2, itot+1) for ux and (jtot+2, itot+2)
for uy, p, psi and temp, halo rows included.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBORACLE = os.path.join(HERE, "build", "liboracle.so")
LIBREF = os.path.join(HERE, "_ref", "libsnsref.so")

_P = ctypes.c_void_p
_D = ctypes.c_double
_I = ctypes.c_int


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_P)


@dataclass
class Config:
    itot: int
    jtot: int
    ly: float = 2.0
    stretch: float = 1e9  # >= itot/2 selects the uniform grid (src/param/init.c:148)
    Ra: float = 1e8
    Pr: float = 1.0
    with_temperature: bool = True
    with_thermal_forcing: bool = True


class _Case:
    """Shared helpers; subclasses bind the C entry points."""

    cfg: Config

    def shapes(self):
        c = self.cfg
        return (c.jtot + 2, c.itot + 1), (c.jtot + 2, c.itot + 2)

    def get_state(self):
        su, sc = self.shapes()
        ux, uy, p, psi, t = (np.zeros(su), np.zeros(sc), np.zeros(sc), np.zeros(sc), np.zeros(sc))
        self._get_state(_ptr(ux), _ptr(uy), _ptr(p), _ptr(psi), _ptr(t))
        return {"ux": ux, "uy": uy, "p": p, "psi": psi, "temp": t}

    def set_state(self, ux, uy, p, temp):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (ux, uy, p, temp)]
        self._set_state(*[_ptr(a) for a in arrs])

    def get_sources(self):
        c = self.cfg
        sx = np.zeros((c.jtot, c.itot - 1))
        sy = np.zeros((c.jtot, c.itot))
        st = np.zeros((c.jtot, c.itot))
        self._get_sources(_ptr(sx), _ptr(sy), _ptr(st))
        return {"srcuxa": sx, "srcuya": sy, "srctempa": st}

    def get_grid(self):
        c = self.cfg
        xf, xc, dxf, dxc = np.zeros(c.itot + 1), np.zeros(c.itot + 2), np.zeros(c.itot), np.zeros(c.itot + 1)
        dy = _D()
        self._get_grid(_ptr(xf), _ptr(xc), _ptr(dxf), _ptr(dxc), ctypes.byref(dy))
        return {"xf": xf, "xc": xc, "dxf": dxf, "dxc": dxc, "dy": dy.value}

    def get_dt(self):
        dt, ix, iy, t, st = _D(), _I(), _I(), _D(), _I()
        self._get_dt(ctypes.byref(dt), ctypes.byref(ix), ctypes.byref(iy), ctypes.byref(t), ctypes.byref(st))
        return {"dt": dt.value, "implicitx": ix.value, "implicity": iy.value, "time": t.value, "step": st.value}


class OracleCase(_Case):
    """The C restatement (sns_oracle.c)."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            if not os.path.exists(LIBORACLE):
                raise RuntimeError(f"oracle library missing: {LIBORACLE} (run oracle/build.py)")
            lib = ctypes.CDLL(LIBORACLE)
            lib.oracle_create.restype = _P
            lib.oracle_create.argtypes = [_I, _I, _D, _D, _D, _D, _I, _I]
            for name in ("oracle_destroy",):
                getattr(lib, name).argtypes = [_P]
            lib.oracle_set_threads.argtypes = [_I]
            lib.oracle_set_costs.argtypes = [_P, _P]
            lib.oracle_set_dt.argtypes = [_P, _D, _I, _I]
            lib.oracle_set_time.argtypes = [_P, _D, _I]
            lib.oracle_get_dt.argtypes = [_P] + [_P] * 5
            for name in ("oracle_decide_dt", "oracle_update_boundaries"):
                getattr(lib, name).argtypes = [_P]
            for name in ("oracle_substage", "oracle_temperature_force_and_update", "oracle_fluid_update_velocity",
                         "oracle_fluid_compute_potential", "oracle_fluid_correct_velocity",
                         "oracle_fluid_update_pressure"):
                getattr(lib, name).argtypes = [_P, _I]
            lib.oracle_run.argtypes = [_P, _I, _I]
            lib.oracle_get_state.argtypes = [_P] + [_P] * 5
            lib.oracle_set_state.argtypes = [_P] + [_P] * 4
            lib.oracle_get_sources.argtypes = [_P] * 4
            lib.oracle_set_sources.argtypes = [_P] * 4
            lib.oracle_get_grid.argtypes = [_P] * 6
            lib.oracle_diagnostics.argtypes = [_P, _P]
            cls._lib = lib
        return cls._lib

    def __init__(self, cfg: Config, threads: int = 1):
        self.cfg = cfg
        lib = self.lib()
        lib.oracle_set_threads(threads)
        self.h = lib.oracle_create(cfg.itot, cfg.jtot, cfg.ly, cfg.stretch, cfg.Ra, cfg.Pr,
                                   int(cfg.with_temperature), int(cfg.with_thermal_forcing))
        if not self.h:
            raise ValueError(f"oracle rejected configuration {cfg}")

    def close(self):
        if self.h:
            self.lib().oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _get_state(self, *a):
        self.lib().oracle_get_state(self.h, *a)

    def _set_state(self, *a):
        self.lib().oracle_set_state(self.h, *a)

    def _get_sources(self, *a):
        self.lib().oracle_get_sources(self.h, *a)

    def set_sources(self, srcuxa, srcuya, srctempa):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (srcuxa, srcuya, srctempa)]
        self.lib().oracle_set_sources(self.h, *[_ptr(a) for a in arrs])

    def _get_grid(self, *a):
        self.lib().oracle_get_grid(self.h, *a)

    def _get_dt(self, *a):
        self.lib().oracle_get_dt(self.h, *a)

    def set_costs(self, w):
        arr = np.asarray(w, dtype=np.float64)
        self.lib().oracle_set_costs(self.h, _ptr(arr))

    def set_dt(self, dt, implicitx=0, implicity=0):
        self.lib().oracle_set_dt(self.h, dt, implicitx, implicity)

    def set_time(self, time, step):
        self.lib().oracle_set_time(self.h, time, step)

    def decide_dt(self):
        self.lib().oracle_decide_dt(self.h)

    def substage(self, rk):
        self.lib().oracle_substage(self.h, rk)

    def run(self, nsteps, decide=True):
        self.lib().oracle_run(self.h, nsteps, int(decide))

    def call(self, name, rk=None):
        fn = getattr(self.lib(), "oracle_" + name)
        return fn(self.h) if rk is None else fn(self.h, rk)

    def diagnostics(self):
        out = np.zeros(11)
        self.lib().oracle_diagnostics(self.h, _ptr(out))
        return out


class RefCase(_Case):
    """The reference's own compiled sources (one instance per process at a time)."""

    _lib = None

    @classmethod
    def available(cls):
        return os.path.exists(LIBREF)

    @classmethod
    def lib(cls):
        if cls._lib is None:
            lib = ctypes.CDLL(LIBREF)
            lib.ref_open.argtypes = [_I, _I, _D, _D, _D, _D, _I, _I, ctypes.c_char_p]
            lib.ref_set_costs.argtypes = [_P]
            lib.ref_set_dt.argtypes = [_D, _I, _I]
            lib.ref_get_dt.argtypes = [_P] * 5
            lib.ref_substage.argtypes = [_I]
            lib.ref_run.argtypes = [_I, _I]
            lib.ref_get_state.argtypes = [_P] * 5
            lib.ref_set_state.argtypes = [_P] * 4
            lib.ref_get_sources.argtypes = [_P] * 3
            lib.ref_get_grid.argtypes = [_P] * 5
            lib.ref_logging.argtypes = [ctypes.c_char_p]
            lib.ref_save.argtypes = [ctypes.c_char_p]
            lib.ref_stats_run.argtypes = [_I, ctypes.c_char_p]
            cls._lib = lib
        return cls._lib

    def __init__(self, cfg: Config, restart_dir: str | None = None):
        self.cfg = cfg
        rc = self.lib().ref_open(cfg.itot, cfg.jtot, cfg.ly, cfg.stretch, cfg.Ra, cfg.Pr,
                                 int(cfg.with_temperature), int(cfg.with_thermal_forcing),
                                 restart_dir.encode() if restart_dir else None)
        if rc != 0:
            raise RuntimeError("reference instance already open in this process")
        self.open = True

    def close(self):
        if self.open:
            self.lib().ref_close()
            self.open = False

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _get_state(self, *a):
        self.lib().ref_get_state(*a)

    def _set_state(self, *a):
        self.lib().ref_set_state(*a)

    def _get_sources(self, *a):
        self.lib().ref_get_sources(*a)

    def _get_grid(self, *a):
        self.lib().ref_get_grid(*a)

    def _get_dt(self, *a):
        self.lib().ref_get_dt(*a)

    def set_costs(self, w):
        arr = np.asarray(w, dtype=np.float64)
        self.lib().ref_set_costs(_ptr(arr))

    def set_dt(self, dt, implicitx=0, implicity=0):
        self.lib().ref_set_dt(dt, implicitx, implicity)

    def decide_dt(self):
        self.lib().ref_decide_dt()

    def substage(self, rk):
        self.lib().ref_substage(rk)

    def run(self, nsteps, decide=True):
        self.lib().ref_run(nsteps, int(decide))

    def logging(self, directory: str):
        os.makedirs(os.path.join(directory, "output", "log"), exist_ok=True)
        return self.lib().ref_logging(directory.encode())

    def stats_run(self, nsteps: int, directory: str):
        """nsteps steps collecting statistics after each, then the reference's
        statistics_output under directory/output/stat"""
        os.makedirs(os.path.join(directory, "output", "stat"), exist_ok=True)
        return self.lib().ref_stats_run(nsteps, directory.encode())

    def save(self, directory: str):
        os.makedirs(os.path.join(directory, "output", "save"), exist_ok=True)
        return self.lib().ref_save(directory.encode())


def parse_ref_log(directory: str) -> np.ndarray:
    """The 11 quantities of oracle_diagnostics, read back from the reference's
    text logs (src/logging.c:75,117,168,267): last line of each file."""
    d = os.path.join(directory, "output", "log")

    def last(name):
        with open(os.path.join(d, name)) as fh:
            return [float(v) for v in fh.read().strip().splitlines()[-1].split()[1:]]

    div = last("divergence.dat")
    mom = last("momentum.dat")
    en = last("energy.dat")
    nu = last("nusselt.dat")
    return np.array(div + mom + en + nu)
