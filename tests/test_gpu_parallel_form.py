"""The plain FP64 path with the Poisson lines and the Crank-Nicolson lines
solved by the partition method and parallel cyclic reduction
(sns_set_form(SNS_FORM_PARALLEL)) against the CPU oracle, whose Thomas
recurrences are the reference's (src/linalg.c:9-108). The two differ by
rounding only, so the bar is the path's stated tolerance: 1e-12 relative L2
per field (ux, uy, T, p) after the stated step counts of the Rayleigh-Benard
workloads.

Also here: the bounded device waits of the fused Poisson launch and of the
parallel tridiagonal launch. A test makes a wait run out (a completion flag
that nothing sets, or a copy that is never issued), checks that the next
synchronising call reports SNS_ERR_STATE, and that the solver then steps on
correctly. No GPU fault is involved: every wait is bounded.
"""
import numpy as np
import pytest

from oracle.bindings import Config, OracleCase

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12
STATE = ("ux", "uy", "p", "temp")


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from simplenavierstokessolver_gb300.build import build

    build()


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def interior(state):
    return {k: state[k][1:-1, 1:-1] for k in STATE}


def _case(cfg, costs=(1, 2, 2, 3)):
    from simplenavierstokessolver_gb300 import Case

    return Case(cfg.itot, cfg.jtot, ly=cfg.ly, stretch=cfg.stretch, Ra=cfg.Ra, Pr=cfg.Pr, costs=list(costs))


def _errors(c, o):
    g, r = interior(c.get_state()), interior(o.get_state())
    return {k: rel_l2(g[k], r[k]) for k in STATE}


@pytest.mark.parametrize("nx,ny", [(256, 128), (64, 32), (2048, 64), (64, 16), (64, 8)],
                         ids=["256x128", "64x32", "2048x64", "64x16", "64x8"])
def test_poisson_solve_alone_matches_oracle(nx, ny):
    """one fluid_compute_potential on a seeded divergent velocity: psi
    within round-off of the Thomas solution (segments of 8, 2 and 64 rows;
    itot 2048 reads its factors from global memory, the others stage them
    in shared memory). The DFTs: radix-8 Stockham passes 8x8 (jtot 128),
    8x2 (32), 8x4 (64), one radix-8 pass (16), and the radix-2/4 stages
    below jtot 16 (8). The mean mode's line is the Neumann Laplacian, whose
    condition number grows as itot^2: two solution methods differ by that
    times the rounding, hence the bound (an indexing fault is O(1))."""
    cfg = Config(nx, ny, ly=1.0, Ra=1e7, Pr=1.0)
    rng = np.random.default_rng(3)
    su, sc = (cfg.jtot + 2, cfg.itot + 1), (cfg.jtot + 2, cfg.itot + 2)
    state = (0.1 * rng.uniform(-1, 1, su), 0.1 * rng.uniform(-1, 1, sc), np.zeros(sc), rng.uniform(-0.5, 0.5, sc))
    o = OracleCase(cfg)
    o.set_state(*state)
    o.call("update_boundaries")
    with _case(cfg) as c:
        c.set_form(True)
        c.set_state(*state)
        for x in (c, o):
            x.set_dt(1e-3, 0, 0)
        for rk in range(3):
            c.fluid_compute_potential(rk)
            o.call("fluid_compute_potential", rk)
            err = rel_l2(c.get_state()["psi"][1:-1, 1:-1], o.get_state()["psi"][1:-1, 1:-1])
            assert err < 1e-10, (rk, err)


@pytest.mark.parametrize("nx,ny,Ra,steps", [(128, 256, 1e8, 1000), (512, 1024, 1e9, 2000)],
                         ids=["128x256_1000_steps", "512x1024_2000_steps"])
def test_rayleigh_benard_within_tolerance(nx, ny, Ra, steps):
    cfg = Config(nx, ny, ly=2.0, Ra=Ra, Pr=1.0)
    o = OracleCase(cfg, threads=16)
    o.set_costs([1, 2, 2, 3])
    with _case(cfg) as c:
        c.set_form(True)
        done = 0
        while done < steps:
            k = min(500, steps - done)
            c.run(k)
            o.run(k)
            done += k
        errs = _errors(c, o)
        print(f"{nx}x{ny} after {steps} steps, relative L2 against the oracle: {errs}")
        assert all(e <= REL_TOL for e in errs.values()), errs
        # dt follows from the velocity, so it agrees to round-off as well
        assert abs(c.get_dt()["dt"] - o.get_dt()["dt"]) <= 1e-12 * o.get_dt()["dt"]
        d_gpu, d_ref = c.diagnostics(), o.diagnostics()
        assert np.allclose(d_gpu[4:], d_ref[4:], rtol=1e-10, atol=0), (d_gpu, d_ref)


@pytest.mark.parametrize("costs", [[1, 2, 2, 3], [4, 3, 2, 1]], ids=["exp_exp", "imp_imp"])
def test_reference_named_calls_within_tolerance(costs):
    cfg = Config(128, 64, ly=1.0, Ra=1e7, Pr=0.8)
    o = OracleCase(cfg)
    o.set_costs(costs)
    with _case(cfg, costs) as c:
        c.set_form(True)
        c.run_calls(20)
        o.run(20)
        errs = _errors(c, o)
        assert all(e <= REL_TOL for e in errs.values()), errs


@pytest.mark.parametrize("scheme", [(1, 0), (0, 1), (1, 1)], ids=["imp_x", "imp_y", "imp_imp"])
@pytest.mark.parametrize("nx,ny", [(64, 128), (256, 64)], ids=["64x128", "256x64"])
def test_crank_nicolson_calls_within_round_off(scheme, nx, ny):
    """The Crank-Nicolson solves of the parallel form (partition method: one
    lane per segment of itot/32 rows along x, of jtot/32 rows along y, whose
    periodic lines give a cyclic interface system) against the oracle's
    Thomas recurrences (src/linalg.c:9-108), call by call on seeded fields
    with non-zero previous sources: segments of 2 and 8 rows along x, 4 and 2
    along y (the form needs the mean mode's last pivot to vanish, which on
    the reference's unit-length x means a power-of-two itot). Each substage
    starts from the oracle's state, and the increments that
    temperature_update_temp and fluid_update_velocity add are compared: a
    wrong coupling anywhere in a line changes them at O(1)."""
    cfg = Config(nx, ny, ly=1.0, Ra=2e5, Pr=0.8)
    rng = np.random.default_rng(17)
    su, sc = (cfg.jtot + 2, cfg.itot + 1), (cfg.jtot + 2, cfg.itot + 2)
    state = (0.2 * rng.uniform(-1, 1, su), 0.2 * rng.uniform(-1, 1, sc), 0.05 * rng.uniform(-1, 1, sc),
             rng.uniform(-0.5, 0.5, sc))
    src = {"srcuxa": rng.uniform(-1, 1, (cfg.jtot, cfg.itot - 1)), "srcuya": rng.uniform(-1, 1, (cfg.jtot, cfg.itot)),
           "srctempa": rng.uniform(-1, 1, (cfg.jtot, cfg.itot))}
    o = OracleCase(cfg)
    o.set_state(*state)
    o.set_sources(src["srcuxa"], src["srcuya"], src["srctempa"])
    o.call("update_boundaries")
    with _case(cfg) as c:
        c.set_form(True)
        c.set_state(*state, sources=src)
        for x in (c, o):
            x.set_dt(2e-3, *scheme)
        for rk in range(3):
            s0 = o.get_state()
            c.temperature_compute_force()
            c.temperature_update_temp(rk)
            o.call("temperature_force_and_update", rk)
            g, r = c.get_state(), o.get_state()
            inc = rel_l2(g["temp"][1:-1, 1:-1] - s0["temp"][1:-1, 1:-1], r["temp"][1:-1, 1:-1] - s0["temp"][1:-1, 1:-1])
            assert inc <= 1e-12, ("temperature increment", rk, inc)
            c.fluid_update_velocity(rk)
            o.call("fluid_update_velocity", rk)
            g, r = c.get_state(), o.get_state()
            for k in ("ux", "uy"):
                inc = rel_l2(g[k][1:-1, 1:-1] - s0[k][1:-1, 1:-1], r[k][1:-1, 1:-1] - s0[k][1:-1, 1:-1])
                assert inc <= 1e-12, (k, "increment", rk, inc)
            for name in ("fluid_compute_potential", "fluid_correct_velocity", "fluid_update_pressure"):
                getattr(c, name)(rk)
                o.call(name, rk)
            # the next substage from the oracle's state
            r, rs = o.get_state(), o.get_sources()
            c.set_state(r["ux"], r["uy"], r["p"], r["temp"], sources=rs)


def test_rayleigh_benard_2048x4096_50_steps_within_tolerance():
    """The 2048 x 4096, Ra 1e10 instance, whose cost table picks
    Crank-Nicolson in x and y: the partition-method solves along both
    directions (segments of 64 and 128 rows) and the parallel Poisson lines,
    50 steps against the oracle."""
    cfg = Config(2048, 4096, ly=2.0, Ra=1e10, Pr=1.0)
    o = OracleCase(cfg, threads=16)
    o.set_costs([1, 2, 2, 3])
    with _case(cfg) as c:
        c.set_form(True)
        c.run(50)
        o.run(50)
        d = c.get_dt()
        assert (d["implicitx"], d["implicity"]) == (1, 1)
        errs = _errors(c, o)
        print(f"2048x4096 after 50 steps, relative L2 against the oracle: {errs}")
        assert all(e <= REL_TOL for e in errs.values()), errs


def test_switching_forms_mid_run():
    """Thomas -> parallel -> Thomas within one run stays within tolerance, and
    the Thomas form alone stays bit for bit"""
    cfg = Config(64, 128, ly=2.0, Ra=1e7, Pr=1.0)
    o = OracleCase(cfg)
    with _case(cfg) as c:
        c.run(10)
        o.run(10)
        assert np.array_equal(c.get_state()["ux"], o.get_state()["ux"])
        c.set_form(True)
        c.run(10)
        c.set_form(False)
        c.run(10)
        o.run(20)
        errs = _errors(c, o)
        assert all(e <= REL_TOL for e in errs.values()), errs


@pytest.mark.parametrize("nx,stretch", [(100, 1e9), (64, 3)], ids=["itot_not_multiple_of_32", "stretched"])
def test_unsupported_grids_are_rejected(nx, stretch):
    from simplenavierstokessolver_gb300 import _native as N

    cfg = Config(nx, 64, ly=1.0, Ra=1e6, Pr=1.0, stretch=stretch)
    with _case(cfg) as c:
        rc = c.lib.sns_set_form(c.fluid, N.SNS_FORM_PARALLEL)
        if rc == N.SNS_OK:
            # a stretched grid whose mean-mode pivot vanishes after all is fine
            assert stretch != 1e9
            return
        assert rc == N.SNS_ERR_UNSUPPORTED
        assert c.lib.sns_get_form(c.fluid) == N.SNS_FORM_EXACT
        c.run(2)  # the Thomas form runs on


def test_fused_launch_wait_runs_out_and_is_reported():
    """The fused Poisson launch's sweep waits for a completion flag that no
    worker writes (stale), gives up after a few polls, and the workers give
    up waiting for the sweep: the call reports SNS_ERR_STATE and names the
    wait; another solver in the same process is unaffected."""
    from simplenavierstokessolver_gb300 import SnsError
    from simplenavierstokessolver_gb300 import _native as N

    cfg = Config(64, 128, ly=2.0, Ra=1e7, Pr=1.0)
    with _case(cfg) as c, _case(cfg) as other:
        c.run(3)
        c.set_wait_limit(64, stale=True)
        with pytest.raises(SnsError) as ei:
            c.run(1)
        assert ei.value.code == N.SNS_ERR_STATE
        assert "gave up" in str(ei.value)
        other.run(5)
        o = OracleCase(cfg)
        o.run(5)
        for k in ("ux", "uy", "p", "psi", "temp"):
            assert np.array_equal(other.get_state()[k], o.get_state()[k]), k


def test_fused_wait_failure_then_three_kernels_match_oracle():
    from simplenavierstokessolver_gb300 import SnsError

    cfg = Config(64, 128, ly=2.0, Ra=1e7, Pr=1.0)
    o = OracleCase(cfg)
    with _case(cfg) as c:
        c.run(3)
        o.run(3)
        h_state, h_src = c.get_state(), c.get_sources()
        clock = c.get_dt()
        c.set_wait_limit(64, stale=True)
        with pytest.raises(SnsError):
            c.run(1)
        c.set_wait_limit(0)
        # restore the state and sources of step 3 and step on (fusing is off now)
        c.set_state(h_state["ux"], h_state["uy"], h_state["p"], h_state["temp"], sources=h_src)
        c.set_time(clock["time"], clock["step"])
        c.run(4)
        o.run(4)
        assert c.get_dt() == o.get_dt()
        for k in ("ux", "uy", "p", "psi", "temp"):
            assert np.array_equal(c.get_state()[k], o.get_state()[k]), k


def test_parallel_tridiagonal_wait_runs_out_and_is_reported():
    """The parallel tridiagonal launch issues no copy (stale): each warp's
    bounded wait on its mbarrier runs out, the launch ends, the call reports
    SNS_ERR_STATE; the next steps (copies issued again) are correct."""
    from simplenavierstokessolver_gb300 import SnsError
    from simplenavierstokessolver_gb300 import _native as N

    cfg = Config(64, 128, ly=2.0, Ra=1e7, Pr=1.0)
    o = OracleCase(cfg)
    with _case(cfg) as c:
        c.set_form(True)
        c.run(3)
        o.run(3)
        h_state, h_src = c.get_state(), c.get_sources()
        clock = c.get_dt()
        c.set_wait_limit(256, stale=True)
        with pytest.raises(SnsError) as ei:
            c.run(1)
        assert ei.value.code == N.SNS_ERR_STATE
        c.set_wait_limit(0)
        c.set_state(h_state["ux"], h_state["uy"], h_state["p"], h_state["temp"], sources=h_src)
        c.set_time(clock["time"], clock["step"])
        c.run(4)
        o.run(4)
        errs = _errors(c, o)
        assert all(e <= REL_TOL for e in errs.values()), errs
