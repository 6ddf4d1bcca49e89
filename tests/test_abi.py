"""CPU-side checks of the C ABI (no GPU): the library loads, exports every
symbol include/*.h declares, its struct layouts agree with the bindings, and
its host-only logic (grid set-up, boundary rules, argument validation)
matches the oracle bit for bit."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from oracle.bindings import Config, OracleCase

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def native():
    from simplenavierstokessolver_gb300.build import build

    build()
    from simplenavierstokessolver_gb300 import _native

    return _native


def declared_symbols():
    names = set()
    for path in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(path).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"extern\s+[^;(]*?\b(\w+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_every_declared_symbol_is_exported(native):
    lib = native.lib()
    names = declared_symbols()
    assert len(names) >= 25
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    # and the bindings cover the same set
    assert names <= set(native.PROTOTYPES), sorted(names - set(native.PROTOTYPES))


def test_struct_layout_matches_bindings(native):
    lib = native.lib()
    out = (ctypes.c_size_t * 32)()
    n = lib.sns_abi_layout(out, 32)
    P = native.Param
    expect = [ctypes.sizeof(P), P.itot.offset, P.dy.offset, P.rkcoefs.offset, P.time.offset, P.dt.offset,
              P.step.offset, P.expimp_wtimes.offset, P.timemax.offset, getattr(P, "log").offset, P.stat.offset,
              ctypes.sizeof(native.Parallel), ctypes.sizeof(native.Fluid), native.Fluid.srcuyg.offset,
              ctypes.sizeof(native.Temperature), ctypes.sizeof(native.CaseDesc), native.CaseDesc.fixed_dt.offset,
              native.CaseDesc.compensated.offset]
    assert n == len(expect)
    assert list(out[:n]) == expect


@pytest.mark.parametrize("itot,jtot,ly,stretch", [(32, 64, 2.0, 1e9), (17, 32, 1.5, 3), (64, 16, 0.5, 0), (5, 8, 2.0, 2)])
def test_param_create_grid_matches_oracle(native, itot, jtot, ly, stretch):
    lib = native.lib()
    p = lib.sns_param_create(itot, jtot, ly, stretch, 1e6, 0.7, 1, 1)
    try:
        pc = p.contents
        o = OracleCase(Config(itot, jtot, ly=ly, stretch=stretch, Ra=1e6, Pr=0.7))
        g = o.get_grid()
        assert np.array_equal(np.ctypeslib.as_array(pc.xf, (itot + 1,)), g["xf"])
        assert np.array_equal(np.ctypeslib.as_array(pc.xc, (itot + 2,)), g["xc"])
        assert np.array_equal(np.ctypeslib.as_array(pc.dxf, (itot,)), g["dxf"])
        assert np.array_equal(np.ctypeslib.as_array(pc.dxc, (itot + 1,)), g["dxc"])
        assert pc.dy == g["dy"]
        # RK coefficients of src/param/init.c:197-213
        a = [pc.rkcoefs[k].alpha for k in range(3)]
        b = [pc.rkcoefs[k].beta for k in range(3)]
        assert a == [32. / 60., 25. / 60., 45. / 60.] and b == [0. / 60., -17. / 60., -25. / 60.]
        assert [pc.rkcoefs[k].gamma for k in range(3)] == [a[k] + b[k] for k in range(3)]
    finally:
        lib.sns_param_destroy(p)


def test_boundary_rules_match_oracle(native):
    lib = native.lib()
    itot, jtot = 12, 8
    cfg = Config(itot, jtot, stretch=2)
    rng = np.random.default_rng(7)
    ux = rng.standard_normal((jtot + 2, itot + 1))
    uy = rng.standard_normal((jtot + 2, itot + 2))
    p = rng.standard_normal((jtot + 2, itot + 2))
    t = rng.standard_normal((jtot + 2, itot + 2))
    o = OracleCase(cfg)
    o.set_state(ux, uy, p, t)
    o.call("update_boundaries")
    ref = o.get_state()
    param = lib.sns_param_create(itot, jtot, 2.0, 2, 1e8, 1.0, 1, 1)
    par = native.Parallel(1, 0, 0, 0)
    try:
        arrs = {k: np.ascontiguousarray(v.copy()) for k, v in (("ux", ux), ("uy", uy), ("p", p), ("temp", t))}
        ptr = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
        assert lib.fluid_update_boundaries_ux(param, ctypes.byref(par), ptr(arrs["ux"])) == 0
        assert lib.fluid_update_boundaries_uy(param, ctypes.byref(par), ptr(arrs["uy"])) == 0
        assert lib.fluid_update_boundaries_p(param, ctypes.byref(par), ptr(arrs["p"])) == 0
        assert lib.temperature_update_boundaries_temp(param, ctypes.byref(par), ptr(arrs["temp"])) == 0
        for k in arrs:
            assert np.array_equal(arrs[k], ref[k]), k
    finally:
        lib.sns_param_destroy(param)


def test_argument_validation_before_any_device_call(native):
    lib = native.lib()
    par2 = native.Parallel(2, 0, 1, 1)
    par1 = native.Parallel(1, 0, 0, 0)
    p = lib.sns_param_create(16, 32, 2.0, 1e9, 1e8, 1.0, 1, 1)
    q = lib.sns_param_create(16, 48, 2.0, 1e9, 1e8, 1.0, 1, 1)
    try:
        assert not lib.fluid_init(p, ctypes.byref(par2))
        assert "single-rank" in native.last_error()
        assert not lib.temperature_init(q, ctypes.byref(par1))
        assert "power of two" in native.last_error()
        assert lib.fluid_update_velocity(p, ctypes.byref(par1), 0, None, None) == native.SNS_ERR_ARG
        assert lib.fluid_update_velocity(p, ctypes.byref(par1), 5, None, None) == native.SNS_ERR_ARG
        assert lib.param_decide_dt(p, ctypes.byref(par1), None) == native.SNS_ERR_ARG
        assert lib.fluid_finalise(None) == native.SNS_ERR_ARG
        assert lib.sns_sync_to_host(None, None, None) == native.SNS_ERR_ARG
    finally:
        lib.sns_param_destroy(p)
        lib.sns_param_destroy(q)


def test_batch_case_footprint(native):
    """sns_batch_case_bytes (host-only): a compensated case also keeps the
    low words of its three previous right-hand sides, one 256-byte aligned
    FP32 field each; unsupported sizes report 0"""
    from simplenavierstokessolver_gb300.batch import Desc, case_bytes

    for nx, ny in ((64, 128), (96, 64), (512, 1024)):
        plain = case_bytes(Desc(nx, ny))
        comp = case_bytes(Desc(nx, ny, compensated=True))
        field = (nx * ny * 4 + 255) // 256 * 256
        assert plain > 0 and comp - plain == 3 * field, (nx, ny, plain, comp)
    assert case_bytes(Desc(64, 100)) == 0  # jtot not a power of two
    assert case_bytes(Desc(40, 128)) == 0  # itot not a multiple of 32
