"""sns_diagnostics_static: the allocation-free diagnostics entry point.

Some callers of this library cannot allocate: a thread that samples a run
while its kernels are in flight (cudaMalloc and cudaFree may synchronise the
device and stall the solver) and a process whose device memory is committed
to a batch arena (an allocation there fails). This entry point serves them
from a fixed scratch array in the library.

Called through the C ABI and compared with sns_diagnostics on the same device
state, two calls in a row and once more after the state moved on: the two
entry points run the same compensated sums in the same order, so their
results are equal bit for bit. The library's allocation counter
(sns_allocations) must not move across the calls.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from simplenavierstokessolver_gb300.build import build

    build()


def _call(case, name):
    from simplenavierstokessolver_gb300 import _native as N

    out = np.full(11, np.nan)
    rc = getattr(case.lib, name)(case.param, case.fluid, case.temperature,
                                 out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    N.check(rc, name)
    return out


@pytest.mark.parametrize("cfg", [dict(itot=128, jtot=256, Ra=1e8, Pr=1.0),
                                 dict(itot=48, jtot=64, ly=1.0, stretch=3.0, Ra=1e6, Pr=0.7)],
                         ids=["uniform_128x256", "stretched_48x64"])
def test_static_scratch_matches_the_allocating_entry_point(cfg):
    from simplenavierstokessolver_gb300.solver import Case

    with Case(**cfg) as c:
        c.run(20)
        ref = _call(c, "sns_diagnostics")  # its first call allocates its partials
        allocs = c.lib.sns_allocations()
        first = _call(c, "sns_diagnostics_static")
        second = _call(c, "sns_diagnostics_static")
        assert c.lib.sns_allocations() == allocs, "sns_diagnostics_static allocated"
        c.run(3)  # the state moves on: the scratch holds nothing stale
        ref2 = _call(c, "sns_diagnostics")
        allocs = c.lib.sns_allocations()
        third = _call(c, "sns_diagnostics_static")
        assert c.lib.sns_allocations() == allocs, "sns_diagnostics_static allocated"
    assert np.all(np.isfinite(ref)) and ref[8] > 1.0
    for got in (first, second):
        assert np.array_equal(got, ref), (got, ref)
    assert np.array_equal(third, ref2), (third, ref2)


def test_grids_beyond_the_scratch_are_rejected():
    from simplenavierstokessolver_gb300 import _native as N
    from simplenavierstokessolver_gb300.solver import Case

    with Case(1024, 4096, Ra=1e8, Pr=1.0) as c:  # 17 x 256 = 4352 block partials > 4096
        with pytest.raises(N.SnsError) as e:
            _call(c, "sns_diagnostics_static")
        assert e.value.code == N.SNS_ERR_UNSUPPORTED
        assert "static" in str(e.value) and "4096" in str(e.value)
        assert np.isfinite(_call(c, "sns_diagnostics")).all()  # the allocating form still serves it
