"""The deterministic cost model that replaces param_estimate_cost's wall-clock
emulation (src/param/estimate_cost.c:44-74). Host only."""
import pytest


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from simplenavierstokessolver_gb300.build import build

    build()


def test_model_is_deterministic_and_ordered():
    from simplenavierstokessolver_gb300.solver import cost_model

    for nx, ny in ((128, 256), (512, 1024), (2048, 4096)):
        a = cost_model(nx, ny)
        assert a == cost_model(nx, ny)
        exp, impx, impy, impimp = a
        assert 0 < exp < impx < impimp and exp < impy < impimp
    # larger grids cost more; a slower clock costs more
    assert cost_model(1024, 2048)[0] > cost_model(512, 1024)[0]
    assert cost_model(512, 1024, clock_ghz=1.0)[0] > cost_model(512, 1024)[0]


def test_model_rejects_bad_input():
    from simplenavierstokessolver_gb300 import _native as N
    from simplenavierstokessolver_gb300.solver import cost_model

    with pytest.raises(N.SnsError):
        cost_model(1, 64)
    with pytest.raises(N.SnsError):
        cost_model(64, 64, sm_count=0)
