"""The cost model against CUDA-event timings of the same substages on the
device (the reference's emulate()); param_estimate_cost fills the table that
param_decide_dt reads."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from simplenavierstokessolver_gb300.build import build

    build()


@pytest.mark.parametrize("nx,ny", [(256, 512), (512, 1024), (1024, 2048)])
def test_model_tracks_measured_costs(nx, ny):
    from simplenavierstokessolver_gb300.solver import Case

    with Case(nx, ny, Ra=1e9, Pr=1.0) as c:
        model = c.estimate_cost()
        measured = c.measure_cost(reps=10)
    ratio = np.array(model) / np.array(measured)
    assert np.all((ratio > 0.4) & (ratio < 2.5)), (model, measured)
    # where the measurement separates two treatments clearly, the model orders them the same way
    for a in range(4):
        for b in range(4):
            if measured[a] < 0.75 * measured[b]:
                assert model[a] < model[b], (a, b, model, measured)


def test_estimated_costs_drive_decide_dt():
    """param_decide_dt with the modelled table picks what the reference's
    rule picks with the same table (the oracle restates it)"""
    from oracle.bindings import Config, OracleCase
    from simplenavierstokessolver_gb300.solver import Case

    for nx, ny, ra in ((512, 1024, 1e9), (1024, 2048, 1e10)):
        with Case(nx, ny, Ra=ra, Pr=1.0) as c:
            w = c.estimate_cost()
            c.param_decide_dt()
            d = c.get_dt()
        o = OracleCase(Config(nx, ny, Ra=ra, Pr=1.0))
        o.set_costs(w)
        o.decide_dt()
        od = o.get_dt()
        assert (d["dt"], d["implicitx"], d["implicity"]) == (od["dt"], od["implicitx"], od["implicity"])
