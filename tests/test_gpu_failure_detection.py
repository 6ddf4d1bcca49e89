"""Failure detection without faulting the GPU.

Non-finite state: the reference has no NaN check (its dt rule ignores NaN,
src/param/decide_dt.c:38,46), so a diverged run keeps stepping. Here every
max-|u| reduction also flags a NaN or infinity in ux, uy or p: the plain
path returns SNS_ERR_NONFINITE from param_decide_dt (after deciding dt as
the reference would) and sns_run stops stepping; a batched case is flagged
by its own correction kernel and reported by sns_batch_case_status, while
the other cases of the batch step on unaffected. The failures are seeded
from the host.

Bounded waits of the batched tridiagonal launch: a step that issues no
bulk copy (stale) makes every mbarrier wait run out; sns_batch_synchronize
reports SNS_ERR_STATE from this batch's own error word, and the next steps
are correct.
"""
import numpy as np
import pytest

from oracle.bindings import Config, OracleCase

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from simplenavierstokessolver_gb300.build import build

    build()


def _case(cfg, costs=(1, 2, 2, 3)):
    from simplenavierstokessolver_gb300 import Case

    return Case(cfg.itot, cfg.jtot, ly=cfg.ly, stretch=cfg.stretch, Ra=cfg.Ra, Pr=cfg.Pr, costs=list(costs))


@pytest.mark.parametrize("form", ["exact", "parallel"])
@pytest.mark.parametrize("field,value", [("ux", np.nan), ("uy", np.inf), ("p", np.nan)])
def test_plain_nonfinite_velocity_or_pressure_is_reported(form, field, value):
    from simplenavierstokessolver_gb300 import SnsError
    from simplenavierstokessolver_gb300 import _native as N

    cfg = Config(64, 64, ly=1.0, Ra=1e6, Pr=1.0)
    with _case(cfg) as c:
        c.set_form(form == "parallel")
        c.run(3)
        s = c.get_state()
        s[field][10, 20] = value
        c.set_state(s["ux"], s["uy"], s["p"], s["temp"])
        step0 = c.get_dt()["step"]
        with pytest.raises(SnsError) as ei:
            c.run(5)
        assert ei.value.code == N.SNS_ERR_NONFINITE
        assert "NaN or infinity" in str(ei.value)
        # sns_run stopped stepping within one step of the seeded value
        assert c.get_dt()["step"] <= step0 + 1


def test_param_decide_dt_reports_and_still_decides_like_the_reference():
    """the dt chosen for a state holding a NaN is the reference's (NaN is
    ignored by its max), and the status says the state is not finite"""
    from simplenavierstokessolver_gb300 import _native as N

    cfg = Config(48, 64, ly=1.0, Ra=1e6, Pr=1.0)
    o = OracleCase(cfg)
    with _case(cfg) as c:
        c.run(2)
        o.run(2)
        s = c.get_state()
        s["ux"][5, 7] = np.nan
        c.set_state(s["ux"], s["uy"], s["p"], s["temp"])
        o.set_state(s["ux"], s["uy"], s["p"], s["temp"])
        rc = c.lib.param_decide_dt(c.param, c.parallel, c.fluid)
        assert rc == N.SNS_ERR_NONFINITE
        o.decide_dt()
        assert c.get_dt()["dt"] == o.get_dt()["dt"]


def test_plain_nonfinite_temperature_reaches_the_velocity_within_a_step():
    from simplenavierstokessolver_gb300 import SnsError
    from simplenavierstokessolver_gb300 import _native as N

    cfg = Config(64, 64, ly=1.0, Ra=1e6, Pr=1.0)
    with _case(cfg) as c:
        c.run(2)
        s = c.get_state()
        s["temp"][12, 30] = np.inf
        c.set_state(s["ux"], s["uy"], s["p"], s["temp"])
        with pytest.raises(SnsError) as ei:
            c.run(3)
        assert ei.value.code == N.SNS_ERR_NONFINITE


def test_finite_runs_report_nothing():
    cfg = Config(64, 128, ly=2.0, Ra=1e8, Pr=1.0)
    with _case(cfg) as c:
        c.run(50)
        c.param_decide_dt()  # raises on a non-zero status


def test_batched_nonfinite_case_is_flagged_and_others_unaffected():
    from simplenavierstokessolver_gb300.batch import Batch, Desc, initial_temperature

    good = Desc(64, 128, ly=2.0, Ra=1e6, Pr=1.0, seed=3, fixed_dt=1e-3)
    bad = Desc(64, 128, ly=2.0, Ra=1e6, Pr=1.0, seed=4, fixed_dt=1e-3)
    t_bad = initial_temperature(bad)
    t_bad[20, 10] = np.nan
    with Batch(256 << 20) as b:
        sg = b.add(good)
        sb = b.add(bad, temp_init=t_bad)
        b.step(4)
        b.synchronize()
        assert b.status(sg)["finite"]
        assert not b.status(sb)["finite"]
        mixed = b.state(sg)
    with Batch(128 << 20) as b:
        s = b.add(good)
        b.step(4)
        alone = b.state(s)
    for k in ("ux", "uy", "p", "temp"):
        assert np.array_equal(mixed[k], alone[k]), k


def test_batched_tridiagonal_wait_runs_out_and_is_reported():
    from simplenavierstokessolver_gb300 import SnsError
    from simplenavierstokessolver_gb300 import _native as N
    from simplenavierstokessolver_gb300.batch import Batch, Desc

    d = Desc(64, 128, ly=2.0, Ra=1e6, Pr=1.0, seed=5, fixed_dt=1e-3)
    with Batch(256 << 20) as b, Batch(128 << 20) as ref:
        s = b.add(d)
        r = ref.add(d)
        b.step(2)
        ref.step(2)
        b.synchronize()
        snapshot = b.state(s)
        b.set_wait_limit(64, stale=True)
        b.step(1)
        with pytest.raises(SnsError) as ei:
            b.synchronize()
        assert ei.value.code == N.SNS_ERR_STATE
        # the other batch's error word is its own: nothing to report there
        ref.synchronize()
        b.set_wait_limit(0)
        b.step(1)
        b.synchronize()  # clean again
        assert np.all(np.isfinite(snapshot["ux"]))
