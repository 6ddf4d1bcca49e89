"""Parity of the plain FP64 GPU path with the CPU oracle at the stated step
counts of the Rayleigh-Benard workloads:

* 128 x 256, Ra 1e8, Pr 1: 1000 steps, both through the fused step
  (sns_run) and through the reference-named calls that the reference's own
  integrate() issues (src/main.c:79-101);
* 512 x 1024, Ra 1e9, Pr 1: 2000 steps (sns_run);
* 2048 x 4096, Ra 1e10, Pr 1: 50 steps (sns_run; the cost table picks
  Crank-Nicolson in x and y there).

Each run starts from the reference's initial condition (srand(0) noise) and
must equal the oracle bit for bit in every field and in dt, which is
stronger than the 1e-12 relative L2 bar the path is specified to. At the end
the reference's log quantities (src/logging.c:36-272) are checked: the mass
balance (divergence of the projected velocity at round-off), and the
divergence, momentum, energy and four Nusselt-number values computed on the
device (sns_diagnostics, compensated sums) against the oracle's sequential
sums of the same state.
"""
import numpy as np
import pytest

from oracle.bindings import Config, OracleCase

pytestmark = pytest.mark.gpu

FIELDS = ("ux", "uy", "p", "psi", "temp")


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from simplenavierstokessolver_gb300.build import build

    build()


def _case(cfg):
    from simplenavierstokessolver_gb300 import Case

    return Case(cfg.itot, cfg.jtot, ly=cfg.ly, stretch=cfg.stretch, Ra=cfg.Ra, Pr=cfg.Pr, costs=[1, 2, 2, 3])


def _check_balances(c, o, cfg, what):
    state = c.get_state()
    ref = o.get_state()
    bad = {k: float(np.abs(state[k] - ref[k]).max()) for k in FIELDS if not np.array_equal(state[k], ref[k])}
    assert not bad, f"{what}: differs from the oracle: {bad}"
    assert c.get_dt() == o.get_dt(), what
    d_ref = o.diagnostics()
    d_gpu = c.diagnostics()
    # mass balance: the largest cell divergence is round-off of the velocity
    # differences it is formed from (|u| / spacing times a few ulps)
    umax = max(np.abs(state["ux"]).max(), np.abs(state["uy"]).max())
    spacing = min(1.0 / cfg.itot, cfg.ly / cfg.jtot)
    assert d_ref[0] <= 64 * np.finfo(float).eps * umax / spacing, (what, d_ref[0], umax)
    assert abs(d_ref[1]) <= 64 * np.finfo(float).eps * umax / spacing * cfg.itot * cfg.jtot, (what, d_ref[1])
    # the device's compensated sums against the reference's sequential ones
    assert d_gpu[0] == d_ref[0], what
    atol = np.zeros(9)
    atol[:2] = 1e-14 * max(1.0, umax)  # momenta: signed sums that cancel
    scale = np.maximum(np.abs(d_ref[2:]), 1e-12)
    assert np.all(np.abs(d_gpu[2:] - d_ref[2:]) <= 1e-12 * scale + atol), (what, d_gpu, d_ref)
    # the four Nusselt numbers are finite and positive (they agree with each
    # other only as time averages of a statistically steady flow)
    assert np.all(np.isfinite(d_gpu[7:])) and np.all(d_gpu[7:] > 0), (what, d_gpu[7:])


@pytest.mark.parametrize("calls", [False, True], ids=["fused_run", "reference_calls"])
def test_rayleigh_benard_128x256_1000_steps(calls):
    cfg = Config(128, 256, ly=2.0, Ra=1e8, Pr=1.0)
    o = OracleCase(cfg, threads=16)
    o.set_costs([1, 2, 2, 3])
    with _case(cfg) as c:
        if calls:
            c.run_calls(1000)
        else:
            c.run(1000)
        o.run(1000)
        _check_balances(c, o, cfg, "128x256 after 1000 steps")


def test_rayleigh_benard_512x1024_2000_steps():
    cfg = Config(512, 1024, ly=2.0, Ra=1e9, Pr=1.0)
    o = OracleCase(cfg, threads=16)
    o.set_costs([1, 2, 2, 3])
    with _case(cfg) as c:
        # in slices, so that a divergence is reported with the step it appeared at
        for _ in range(4):
            c.run(500)
            o.run(500)
            assert c.get_dt() == o.get_dt()
        _check_balances(c, o, cfg, "512x1024 after 2000 steps")


def test_rayleigh_benard_2048x4096_50_steps():
    cfg = Config(2048, 4096, ly=2.0, Ra=1e10, Pr=1.0)
    o = OracleCase(cfg, threads=16)
    o.set_costs([1, 2, 2, 3])
    with _case(cfg) as c:
        c.run(50)
        o.run(50)
        dt = c.get_dt()
        assert (dt["implicitx"], dt["implicity"]) == (1, 1)
        _check_balances(c, o, cfg, "2048x4096 after 50 steps")
