"""Parity of the plain FP64 GPU path (through the C ABI) with the CPU oracle
and with the golden fixtures recorded from the reference.

The GPU path and the oracle built on the same host share every host-side
input (grid, eigenvalues, twiddles from the same libm), so they must agree
bit for bit (np.array_equal, which equates +0 and -0). Against the fixtures
recorded on another host the tolerance is 1e-12 relative L2 per field (the
host libm may differ in the last bit), which is also the bar the path is
specified to meet against the reference.
"""
import json
import os
import platform

import numpy as np
import pytest

from oracle.bindings import Config, OracleCase

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")
MANIFEST = json.load(open(os.path.join(GOLD, "manifest.json")))
FIELDS = ("ux", "uy", "p", "psi", "temp")
REL_TOL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from simplenavierstokessolver_gb300.build import build

    build()


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def gpu_case(cfg: Config, costs):
    from simplenavierstokessolver_gb300 import Case

    return Case(cfg.itot, cfg.jtot, ly=cfg.ly, stretch=cfg.stretch, Ra=cfg.Ra, Pr=cfg.Pr,
                with_temperature=cfg.with_temperature, with_thermal_forcing=cfg.with_thermal_forcing, costs=costs)


def assert_bitwise(a: dict, b: dict, keys, what=""):
    bad = {k: float(np.abs(a[k] - b[k]).max()) for k in keys if not np.array_equal(a[k], b[k])}
    assert not bad, f"{what} differs from the oracle: {bad}"


@pytest.mark.parametrize("fused", [False, True], ids=["reference_calls", "fused_run"])
@pytest.mark.parametrize("name", sorted(MANIFEST))
def test_golden_cases(name, fused):
    meta = MANIFEST[name]
    cfg = Config(**meta["config"])
    g = np.load(os.path.join(GOLD, f"{name}.npz"))
    o = OracleCase(cfg, threads=4)
    o.set_costs(meta["costs"])
    with gpu_case(cfg, meta["costs"]) as c:
        if meta["seeded"]:
            for x in (o, c):
                x.set_state(g["init_ux"], g["init_uy"], g["init_p"], g["init_temp"])
            # seeded arrays carry arbitrary halo values; the reference overwrites
            # them at the first boundary call of the first substage
            o.call("update_boundaries")
        # with the temperature uncoupled the reference never applies its wall
        # and halo rules to it, so only its interior is defined
        fields = FIELDS if cfg.with_temperature else ("ux", "uy", "p", "psi")
        assert_bitwise(c.get_state(), o.get_state(), [k for k in fields if k != "psi"], "initial state")
        if fused:
            c.run(meta["steps"])
        else:
            c.run_calls(meta["steps"])
        o.run(meta["steps"])
        sg, so = c.get_state(), o.get_state()
        assert c.get_dt() == o.get_dt()
        assert_bitwise(sg, so, fields, name)
        assert np.array_equal(sg["temp"][1:-1, 1:-1], so["temp"][1:-1, 1:-1])
        assert_bitwise(c.get_sources(), o.get_sources(), ("srcuxa", "srcuya", "srctempa"), name)
        for k in fields:
            err = rel_l2(sg[k], g[f"final_{k}"])
            assert err <= REL_TOL or (platform.machine() == "x86_64" and np.array_equal(sg[k], g[f"final_{k}"])), \
                f"{k}: rel L2 {err:.3e} vs the reference's fixture"


@pytest.mark.parametrize("costs", [[1, 2, 2, 3], [3, 1, 4, 5], [3, 4, 1, 5], [4, 3, 2, 1]],
                         ids=["exp_exp", "imp_x", "imp_y", "imp_imp"])
@pytest.mark.parametrize("stretch", [1e9, 3], ids=["uniform", "stretched"])
def test_each_hot_path_call_matches(costs, stretch):
    """Every reference-named call, one at a time, on seeded non-trivial fields
    with non-zero previous RK sources, compared after each call."""
    cfg = Config(24, 32, ly=1.5, Ra=2e5, Pr=0.8, stretch=stretch)
    rng = np.random.default_rng(11)
    su, sc = (cfg.jtot + 2, cfg.itot + 1), (cfg.jtot + 2, cfg.itot + 2)
    state = (0.2 * rng.uniform(-1, 1, su), 0.2 * rng.uniform(-1, 1, sc), 0.05 * rng.uniform(-1, 1, sc),
             rng.uniform(-0.5, 0.5, sc))
    src = {"srcuxa": rng.uniform(-1, 1, (cfg.jtot, cfg.itot - 1)), "srcuya": rng.uniform(-1, 1, (cfg.jtot, cfg.itot)),
           "srctempa": rng.uniform(-1, 1, (cfg.jtot, cfg.itot))}
    o = OracleCase(cfg)
    o.set_costs(costs)
    o.set_state(*state)
    o.set_sources(src["srcuxa"], src["srcuya"], src["srctempa"])
    with gpu_case(cfg, costs) as c:
        c.set_state(*state, sources=src)
        o.call("update_boundaries")
        o.decide_dt()
        c.param_decide_dt()
        assert c.get_dt() == o.get_dt()
        for rk in range(3):
            c.temperature_compute_force()
            c.temperature_update_temp(rk)
            o.call("temperature_force_and_update", rk)
            assert_bitwise(c.get_state(), o.get_state(), ("temp",), f"temperature_update_temp rk={rk}")
            c.fluid_update_velocity(rk)
            o.call("fluid_update_velocity", rk)
            assert_bitwise(c.get_state(), o.get_state(), ("ux", "uy"), f"fluid_update_velocity rk={rk}")
            assert_bitwise(c.get_sources(), o.get_sources(), ("srcuxa", "srcuya", "srctempa"), f"sources rk={rk}")
            c.fluid_compute_potential(rk)
            o.call("fluid_compute_potential", rk)
            assert_bitwise(c.get_state(), o.get_state(), ("psi",), f"fluid_compute_potential rk={rk}")
            c.fluid_correct_velocity(rk)
            o.call("fluid_correct_velocity", rk)
            assert_bitwise(c.get_state(), o.get_state(), ("ux", "uy"), f"fluid_correct_velocity rk={rk}")
            c.fluid_update_pressure(rk)
            o.call("fluid_update_pressure", rk)
            assert_bitwise(c.get_state(), o.get_state(), ("p",), f"fluid_update_pressure rk={rk}")


@pytest.mark.parametrize("implicit", [0, 1], ids=["exp_exp", "imp_imp"])
def test_velocity_update_with_extreme_magnitudes(implicit):
    """On a uniform power-of-two grid the velocity and temperature kernels form
    their products by powers of two in integer arithmetic and recompute a row
    with FP64 products when an operand is a subnormal, infinite or beyond
    2^+-958. Seeded fields with exact zeros, subnormals, tiny and huge normals
    must still match the oracle bit for bit."""
    cfg = Config(64, 32, ly=0.5, Ra=2e5, Pr=0.8)
    rng = np.random.default_rng(5)
    su, sc = (cfg.jtot + 2, cfg.itot + 1), (cfg.jtot + 2, cfg.itot + 2)

    def sprinkle(a, huge=False):
        pick = rng.uniform(size=a.shape)
        sign = np.where(rng.uniform(size=a.shape) < 0.5, -1.0, 1.0)
        a[pick < 0.05] = 0.0
        a[(pick >= 0.05) & (pick < 0.07)] = (sign * 5e-320)[(pick >= 0.05) & (pick < 0.07)]
        a[(pick >= 0.07) & (pick < 0.09)] = (sign * 3e-295)[(pick >= 0.07) & (pick < 0.09)]
        a[(pick >= 0.09) & (pick < 0.10)] = (sign * 1e150)[(pick >= 0.09) & (pick < 0.10)]
        if huge:
            a[(pick >= 0.10) & (pick < 0.11)] = (sign * 1e290)[(pick >= 0.10) & (pick < 0.11)]
        return a

    state = (sprinkle(0.2 * rng.uniform(-1, 1, su)), sprinkle(0.2 * rng.uniform(-1, 1, sc)),
             sprinkle(0.05 * rng.uniform(-1, 1, sc), huge=True), sprinkle(rng.uniform(-0.5, 0.5, sc)))
    src = {"srcuxa": sprinkle(rng.uniform(-1, 1, (cfg.jtot, cfg.itot - 1))),
           "srcuya": sprinkle(rng.uniform(-1, 1, (cfg.jtot, cfg.itot))),
           "srctempa": rng.uniform(-1, 1, (cfg.jtot, cfg.itot))}
    o = OracleCase(cfg)
    o.set_state(*state)
    o.set_sources(src["srcuxa"], src["srcuya"], src["srctempa"])
    with gpu_case(cfg, [1, 2, 2, 3]) as c:
        c.set_state(*state, sources=src)
        o.call("update_boundaries")
        # a fixed dt: the huge velocities would make the chosen one vanishingly small
        for x in (c, o):
            x.set_dt(1e-3, implicit, implicit)
        for rk in range(2):
            c.temperature_compute_force()
            c.temperature_update_temp(rk)
            o.call("temperature_force_and_update", rk)
            assert np.array_equal(c.get_state()["temp"], o.get_state()["temp"], equal_nan=True), f"temp after rk={rk}"
            c.fluid_update_velocity(rk)
            o.call("fluid_update_velocity", rk)
            # the huge seeds overflow by the second substage: NaN where the oracle has NaN
            for got, want in ((c.get_state(), o.get_state()), (c.get_sources(), o.get_sources())):
                for k in set(got) & {"ux", "uy", "srcuxa", "srcuya"}:
                    assert np.array_equal(got[k], want[k], equal_nan=True), f"{k} after rk={rk}"


@pytest.mark.parametrize("costs", [[1, 2, 2, 3], [4, 3, 2, 1]], ids=["exp_exp", "imp_imp"])
def test_whole_steps_with_tiny_magnitudes(costs):
    """Whole steps (the fused path: velocity, temperature, Poisson and the
    correction/pressure kernel) from fields with exact zeros, subnormals and
    normals below 2^-958 in every field: the rows that hold them take the
    FP64 products, the others the integer ones, and the result is the
    oracle's bit for bit."""
    cfg = Config(64, 64, ly=1.0, Ra=1e6, Pr=0.8)
    rng = np.random.default_rng(9)
    su, sc = (cfg.jtot + 2, cfg.itot + 1), (cfg.jtot + 2, cfg.itot + 2)

    def sprinkle(a):
        pick = rng.uniform(size=a.shape)
        sign = np.where(rng.uniform(size=a.shape) < 0.5, -1.0, 1.0)
        a[pick < 0.05] = 0.0
        a[(pick >= 0.05) & (pick < 0.08)] = (sign * 5e-320)[(pick >= 0.05) & (pick < 0.08)]
        a[(pick >= 0.08) & (pick < 0.11)] = (sign * 3e-295)[(pick >= 0.08) & (pick < 0.11)]
        return a

    state = (sprinkle(0.2 * rng.uniform(-1, 1, su)), sprinkle(0.2 * rng.uniform(-1, 1, sc)),
             sprinkle(0.05 * rng.uniform(-1, 1, sc)), sprinkle(rng.uniform(-0.5, 0.5, sc)))
    o = OracleCase(cfg)
    o.set_costs(costs)
    o.set_state(*state)
    with gpu_case(cfg, costs) as c:
        c.set_state(*state)
        o.call("update_boundaries")
        c.run(2)
        o.run(2)
        assert c.get_dt() == o.get_dt()
        assert_bitwise(c.get_state(), o.get_state(), FIELDS, "after 2 steps from tiny magnitudes")


def test_rayleigh_benard_128x256_long_run_is_bitwise():
    """The 128x256, Ra=1e8, Pr=1 Rayleigh-Benard case from the reference's own
    initial condition (srand(0)), 300 steps of the fused path."""
    cfg = Config(128, 256, ly=2.0, Ra=1e8, Pr=1.0)
    o = OracleCase(cfg, threads=8)
    with gpu_case(cfg, [1, 2, 2, 3]) as c:
        c.run(300)
        o.run(300)
        assert c.get_dt() == o.get_dt()
        assert_bitwise(c.get_state(), o.get_state(), FIELDS, "128x256 after 300 steps")


def test_rayleigh_benard_512x1024_is_bitwise():
    cfg = Config(512, 1024, ly=2.0, Ra=1e9, Pr=1.0)
    o = OracleCase(cfg, threads=16)
    with gpu_case(cfg, [1, 2, 2, 3]) as c:
        c.run(4)
        o.run(4)
        assert c.get_dt() == o.get_dt()
        assert_bitwise(c.get_state(), o.get_state(), FIELDS, "512x1024 after 4 steps")


def test_rayleigh_benard_2048x4096_implicit_is_bitwise():
    """The largest configuration, 2048 x 4096 at Ra 1e10: the cost table picks
    Crank-Nicolson in x and y (lines of 2048 and 4096), the fused Poisson
    launch runs column groups of two with four sweep warps per block."""
    cfg = Config(2048, 4096, ly=2.0, Ra=1e10, Pr=1.0)
    o = OracleCase(cfg, threads=16)
    with gpu_case(cfg, [1, 2, 2, 3]) as c:
        c.run(2)
        o.run(2)
        dt = c.get_dt()
        assert dt == o.get_dt()
        assert (dt["implicitx"], dt["implicity"]) == (1, 1)
        assert_bitwise(c.get_state(), o.get_state(), FIELDS, "2048x4096 after 2 steps")


def test_divergence_free_and_reference_diagnostics():
    """The projected velocity is solenoidal to round-off (the reference's own
    check, src/logging.c:36-80), and the log quantities computed from the
    synced GPU state equal the oracle's."""
    cfg = Config(64, 128, ly=2.0, Ra=1e7, Pr=1.0)
    o = OracleCase(cfg)
    with gpu_case(cfg, [1, 2, 2, 3]) as c:
        c.run(40)
        o.run(40)
        s = c.get_state()
        check = OracleCase(cfg)
        check.set_state(s["ux"], s["uy"], s["p"], s["temp"])
        d_gpu, d_ref = check.diagnostics(), o.diagnostics()
        assert np.array_equal(d_gpu, d_ref)
        assert d_gpu[0] < 1e-12
        assert abs(d_gpu[1]) < 1e-10


def test_device_diagnostics_match_the_reference_logs():
    """sns_diagnostics (device, compensated sums) against the oracle's
    sequential sums of src/logging.c: equal to the latter's round-off"""
    for cfg in (Config(64, 128, Ra=1e7, Pr=1.0), Config(48, 64, ly=1.0, Ra=1e6, Pr=0.7, stretch=3)):
        o = OracleCase(cfg)
        with gpu_case(cfg, [1, 2, 2, 3]) as c:
            c.run(30)
            o.run(30)
            dg, dr = c.diagnostics(), o.diagnostics()
        assert dg[0] == dr[0]  # the maximum is exact
        # the momenta (2, 3) are sums of signed terms that cancel to ~1e-20:
        # their error is bounded by round-off of the summed magnitudes instead
        atol = np.zeros(9)
        atol[:2] = 1e-16
        scale = np.maximum(np.abs(dr[2:]), 1e-12)
        assert np.all(np.abs(dg[2:] - dr[2:]) <= 1e-12 * scale + atol), (dg, dr)
        assert abs(dg[1] - dr[1]) < 1e-12


def test_restart_through_host_arrays_continues_bitwise():
    """sync_to_host -> sync_to_device round trip (the restart path) changes nothing."""
    cfg = Config(32, 64, Ra=1e8, Pr=1.0)
    o = OracleCase(cfg)
    with gpu_case(cfg, [1, 2, 2, 3]) as c:
        c.run(5)
        o.run(5)
        s = c.get_state()
        c.set_state(s["ux"], s["uy"], s["p"], s["temp"], sources=c.get_sources())
        c.run(5)
        o.run(5)
        assert_bitwise(c.get_state(), o.get_state(), ("ux", "uy", "p", "temp"), "after restart")


@pytest.mark.parametrize("costs", [[1, 2, 2, 3], [4, 3, 2, 1]], ids=["exp_exp", "imp_imp"])
def test_state_only_syncs_around_whole_steps_are_bitwise(costs):
    """sns_sync_state_to_host / _to_device move ux, uy, p and temp alone. The
    state saved after 3 steps and put back after 2 more (the device keeps the
    later psi and sources) continues exactly like the oracle's uninterrupted
    run, and the synced host state equals what the full sync gives."""
    cfg = Config(48, 64, ly=1.5, Ra=1e7, Pr=0.8, stretch=3)
    o = OracleCase(cfg)
    o.set_costs(costs)
    keys = ("ux", "uy", "p", "temp")
    with gpu_case(cfg, costs) as c:
        h = c.host_arrays()
        c.run(3)
        c.sync_state_to_host()
        saved = {k: h[k].copy() for k in keys}
        clock = c.get_dt()
        h["psi"][...] = np.nan  # not touched by the state-only copies
        c.run(2)
        c.sync_state_to_host()
        assert np.isnan(h["psi"]).all()
        assert not np.array_equal(h["ux"], saved["ux"])
        for k in keys:
            h[k][...] = saved[k]
        c.sync_state_to_device()
        c.set_time(clock["time"], clock["step"])
        c.run(4)
        c.sync_state_to_host()
        state = {k: h[k].copy() for k in keys}
        o.run(7)
        full = c.get_state()
        assert c.get_dt() == o.get_dt()
        assert_bitwise(full, o.get_state(), FIELDS, "after a state-only restore")
        for k in keys:
            assert np.array_equal(state[k], full[k]), k


@pytest.mark.parametrize("costs", [[1, 2, 2, 3], [4, 3, 2, 1]], ids=["exp_exp", "imp_imp"])
def test_resident_reduction_across_calls_is_bitwise(costs):
    """The max-|u| reduction the last substage of sns_run / sns_integrate
    leaves on the device stands in for the next call's own while nothing
    changed the velocity in between: single-step sns_run calls,
    param_decide_dt + sns_integrate steps, and reference-named calls and a
    host round trip in between (which must force a fresh reduction) all
    give the oracle's dt and state bit for bit."""
    cfg = Config(48, 64, ly=1.0, Ra=1e7, Pr=0.8, stretch=3)
    o = OracleCase(cfg)
    o.set_costs(costs)
    with gpu_case(cfg, costs) as c:
        for _ in range(3):
            c.run(1)
        for _ in range(3):
            c.param_decide_dt()
            c.integrate()
            c.set_time(c.get_dt()["time"] + c.get_dt()["dt"], c.get_dt()["step"] + 1)
        c.run_calls(2)
        c.run(1)
        s = c.get_state()
        c.set_state(s["ux"], s["uy"], s["p"], s["temp"], sources=c.get_sources())
        c.run(2)
        o.run(11)
        assert c.get_dt() == o.get_dt()
        assert_bitwise(c.get_state(), o.get_state(), FIELDS, "after mixed calls")


def test_deferred_reference_calls_are_flushed_by_other_calls():
    """temperature_update_temp waits for fluid_compute_potential and
    fluid_correct_velocity for fluid_update_pressure (one launch each pair);
    any other call in between performs the waiting work first. Substages with
    diagnostics, host syncs and a fused-mode toggle wedged between the pairs
    give the oracle's state bit for bit."""
    cfg = Config(40, 64, ly=1.0, Ra=1e7, Pr=0.8)
    o = OracleCase(cfg)
    with gpu_case(cfg, [1, 2, 2, 3]) as c:
        for step in range(3):
            c.param_decide_dt()
            for rk in range(3):
                c.update_boundaries()
                c.temperature_compute_force()
                c.temperature_update_temp(rk)
                if rk == 0:
                    c.diagnostics()
                if rk == 1:
                    c.sync_state_to_host()
                c.fluid_update_velocity(rk)
                c.fluid_compute_potential(rk)
                c.fluid_correct_velocity(rk)
                if rk == 2:
                    c.set_fused(step % 2 == 0)
                if rk == 0:
                    c.sync_to_host()
                c.fluid_update_pressure(rk)
            c.p.step += 1
            c.p.time += c.p.dt
        c.set_fused(True)
        o.run(3)
        assert c.get_dt() == o.get_dt()
        assert_bitwise(c.get_state(), o.get_state(), FIELDS, "reference-named calls with calls in between")


def test_state_only_syncs_of_one_structure_and_bad_arguments():
    """Either structure may be NULL (only the other one's state moves); a
    structure of another solver is rejected with SNS_ERR_ARG."""
    from simplenavierstokessolver_gb300 import _native as N

    cfg = Config(32, 32, ly=1.0, Ra=1e6, Pr=1.0)
    with gpu_case(cfg, [1, 2, 2, 3]) as c, gpu_case(cfg, [1, 2, 2, 3]) as other:
        c.run(2)
        full = c.get_state()
        h = c.host_arrays()
        for k in ("ux", "uy", "p", "temp"):
            h[k][...] = 0.0
        N.check(c.lib.sns_sync_state_to_host(c.param, c.fluid, None), "sns_sync_state_to_host")
        assert np.array_equal(h["ux"], full["ux"]) and np.array_equal(h["p"], full["p"])
        assert not h["temp"].any()
        N.check(c.lib.sns_sync_state_to_host(c.param, None, c.temperature), "sns_sync_state_to_host")
        assert np.array_equal(h["temp"], full["temp"])
        # upload the temperature alone: the velocity on the device stays as it was
        h["temp"][...] = 0.25
        N.check(c.lib.sns_sync_state_to_device(c.param, None, c.temperature), "sns_sync_state_to_device")
        s = c.get_state()
        assert np.array_equal(s["ux"], full["ux"]) and np.all(s["temp"][1:-1, 1:-1] == 0.25)
        rc = c.lib.sns_sync_state_to_device(c.param, c.fluid, other.temperature)
        assert rc == N.SNS_ERR_ARG
        rc = c.lib.sns_sync_state_to_host(c.param, c.fluid, ctypes_cast_temperature(other.fluid))
        assert rc == N.SNS_ERR_ARG


def ctypes_cast_temperature(fluid_ptr):
    """a fluid_t pointer passed where a temperature_t is expected"""
    import ctypes

    from simplenavierstokessolver_gb300 import _native as N

    return ctypes.cast(fluid_ptr, ctypes.POINTER(N.Temperature))


@pytest.mark.parametrize("nx,ny,costs", [(64, 128, [1, 2, 2, 3]), (2048, 256, [1, 2, 2, 3]),
                                          (96, 64, [4, 3, 2, 1])], ids=["64x128", "2048x256", "impimp_96x64"])
def test_fused_poisson_equals_three_kernels(nx, ny, costs):
    """the cooperative Poisson(+temperature) launch against the three-kernel
    form, bit for bit, including column groups of two (nx > 1024)"""
    from simplenavierstokessolver_gb300.solver import Case

    states = []
    for fused in (True, False):
        with Case(nx, ny, Ra=1e8, Pr=1.0, costs=costs) as c:
            c.set_fused(fused)
            c.run(4)
            c.fluid_compute_potential(0)  # the reference-named call takes the same path
            states.append(c.get_state())
    for k in states[0]:
        assert np.array_equal(states[0][k], states[1][k]), k


@pytest.mark.parametrize("nx,ny", [(2, 2), (3, 4), (5, 8), (7, 16), (33, 64), (100, 32), (1030, 16)],
                         ids=lambda v: str(v))
def test_small_and_odd_grids(nx, ny):
    """edge sizes: the smallest grids, odd itot, itot not a multiple of the
    warp or of the column groups, jtot = 2 (a one-point complex DFT)"""
    cfg = Config(nx, ny, ly=2.0, Ra=1e4, Pr=1.0)
    o = OracleCase(cfg)
    with gpu_case(cfg, [1, 2, 2, 3]) as c:
        c.run(5)
        o.run(5)
        assert c.get_dt() == o.get_dt()
        assert_bitwise(c.get_state(), o.get_state(), FIELDS, f"{nx}x{ny}")
