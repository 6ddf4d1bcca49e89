"""The seeded synthetic workloads (CPU only): the Python SplitMix64 draws the
same numbers as the library's C generator (the batched form's initial
temperature noise, sns_case_desc.seed), and the 64-case ensemble and the
serving stream stay within their stated distributions and are reproducible
case by case."""
import numpy as np
import pytest

from oracle.bindings import Config, OracleCase


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from simplenavierstokessolver_gb300.build import build

    build()


@pytest.mark.parametrize("nx,ny,seed", [(64, 32, 12345), (96, 16, 20261203 + 7)])
def test_python_generator_matches_the_library_noise(nx, ny, seed):
    from simplenavierstokessolver_gb300.batch import Desc, initial_temperature
    from simplenavierstokessolver_gb300.workloads import SplitMix64

    got = initial_temperature(Desc(nx, ny, ly=2.0, seed=seed))
    xc = OracleCase(Config(nx, ny, ly=2.0)).get_grid()["xc"]
    g = SplitMix64(seed)
    want = np.empty((ny, nx))
    for j in range(ny):  # the library draws row by row, x fastest
        for i in range(nx):
            r = g.uniform() - 0.5
            want[j, i] = (-0.5 - 0.5) * xc[i + 1] + 0.5 + 0.1 * r  # T(x=0) = +0.5, T(x=1) = -0.5
    assert np.array_equal(got[1:-1, 1:-1], want)
    assert np.all(got[1:-1, 0] == 0.5) and np.all(got[1:-1, -1] == -0.5)


def test_ensemble_is_reproducible_and_in_range():
    from simplenavierstokessolver_gb300.workloads import ensemble

    a = ensemble(64)
    assert len(a) == 64
    assert [(d.itot, d.Ra, d.Pr, d.seed) for d in a] == [(d.itot, d.Ra, d.Pr, d.seed) for d in ensemble(64)]
    # case k does not depend on how many cases are drawn
    assert [(d.itot, d.Ra, d.Pr) for d in ensemble(10)] == [(d.itot, d.Ra, d.Pr) for d in a[:10]]
    for d in a:
        assert d.itot in (64, 128, 256) and d.jtot == 2 * d.itot and d.ly == 2.0
        assert 1e6 <= d.Ra <= 1e9 and 0.7 <= d.Pr <= 7.0
    assert len({d.itot for d in a}) == 3  # all three sizes occur
    assert len({d.seed for d in a}) == 64


def test_serving_stream_is_a_poisson_process_within_its_window():
    from simplenavierstokessolver_gb300.workloads import serving_stream

    descs, arrivals = serving_stream(6.0, 600.0)
    assert len(descs) == len(arrivals)
    arr = np.asarray(arrivals)
    assert np.all(np.diff(arr) >= 0) and arr[0] > 0 and arr[-1] <= 600.0
    # about rate x duration requests; exponential gaps with mean 1 / rate
    assert 0.85 * 3600 < len(arr) < 1.15 * 3600
    gaps = np.diff(np.concatenate([[0.0], arr]))
    assert abs(gaps.mean() - 1 / 6.0) < 0.1 / 6.0
    for d in descs:
        assert d.itot in (64, 128, 256, 512) and d.jtot == 2 * d.itot
        assert 1e6 <= d.Ra <= 1e10 and 0.7 <= d.Pr <= 7.0 and 200 <= d.steps <= 2000
    again, arr2 = serving_stream(6.0, 600.0)
    assert arr2 == arrivals and [d.steps for d in again] == [d.steps for d in descs]
