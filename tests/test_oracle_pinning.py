"""Pins the CPU oracle (the C restatement in oracle/sns_oracle.c) to the
reference: against the golden fixtures recorded from the reference's own
compiled sources (tests/golden/make_golden.py), and -- where the reference
tree is mounted -- against a live run of the reference.

On the machine that generated the fixtures the match is bitwise. Elsewhere the
host libm (sin/cos used for the grid, twiddles and Poisson eigenvalues) may
differ in the last bit, so off that machine the comparison allows a relative
L2 error of 1e-12 per field.
"""
import json
import os
import platform

import numpy as np
import pytest

from oracle.bindings import Config, OracleCase, RefCase

GOLD = os.path.join(os.path.dirname(__file__), "golden")
MANIFEST = json.load(open(os.path.join(GOLD, "manifest.json")))
BITWISE = platform.machine() == "x86_64"
REL_TOL = 1e-12


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def assert_same(a, b, what):
    if BITWISE:
        assert np.array_equal(a, b), f"{what}: max |diff| {np.abs(a - b).max():.3e}"
    else:
        assert rel_l2(a, b) <= REL_TOL, f"{what}: rel L2 {rel_l2(a, b):.3e}"


def load(name):
    meta = MANIFEST[name]
    cfg = Config(**meta["config"])
    return meta, cfg, np.load(os.path.join(GOLD, f"{name}.npz"))


@pytest.mark.parametrize("name", sorted(MANIFEST))
def test_oracle_matches_golden(name):
    meta, cfg, g = load(name)
    o = OracleCase(cfg, threads=2)
    o.set_costs(meta["costs"])
    if meta["seeded"]:
        o.set_state(g["init_ux"], g["init_uy"], g["init_p"], g["init_temp"])
    init = o.get_state()
    for k in ("ux", "uy", "p", "temp"):
        assert_same(init[k], g[f"init_{k}"], f"initial {k}")
    grid = o.get_grid()
    for k in ("xf", "xc", "dxf", "dxc"):
        assert_same(grid[k], g[f"grid_{k}"], f"grid {k}")
    o.run(meta["steps"])
    after = o.get_dt()
    assert after["implicitx"] == meta["after"]["implicitx"]
    assert after["implicity"] == meta["after"]["implicity"]
    assert after["step"] == meta["after"]["step"]
    np.testing.assert_allclose(after["dt"], meta["after"]["dt"], rtol=0 if BITWISE else 1e-14)
    final = o.get_state()
    for k in ("ux", "uy", "p", "psi", "temp"):
        assert_same(final[k], g[f"final_{k}"], f"final {k}")
    src = o.get_sources()
    for k in src:
        assert_same(src[k], g[k], k)
    # the reference's log quantities; divergence is printed with 2 digits
    diag = o.diagnostics()
    log = g["log"]
    np.testing.assert_allclose(diag[2:], log[2:], rtol=1e-14, atol=1e-18)
    assert abs(diag[0] - log[0]) <= 0.06 * abs(log[0]) + 1e-300


def test_oracle_thread_count_does_not_change_bits():
    cfg = Config(32, 64, Ra=1e7, Pr=0.7, stretch=4)
    a, b = OracleCase(cfg, threads=1), OracleCase(cfg, threads=4)
    for o in (a, b):
        o.set_costs([4, 3, 2, 1])  # implicit in both directions
        o.run(3)
    sa, sb = a.get_state(), b.get_state()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k


@pytest.mark.skipif(not RefCase.available(), reason="reference build not present (reference tree not mounted)")
@pytest.mark.parametrize("costs", [[1, 2, 2, 3], [3, 1, 4, 5], [3, 4, 1, 5], [4, 3, 2, 1]])
def test_oracle_matches_live_reference(costs):
    cfg = Config(24, 32, ly=1.5, Ra=3e5, Pr=0.9, stretch=4)
    with RefCase(cfg) as ref:
        o = OracleCase(cfg, threads=3)
        ref.set_costs(costs)
        o.set_costs(costs)
        ref.run(12)
        o.run(12)
        sr, so = ref.get_state(), o.get_state()
        for k in sr:
            assert np.array_equal(sr[k], so[k]), k
        assert ref.get_dt() == o.get_dt()


def test_oracle_rejects_unsupported_lengths():
    with pytest.raises(ValueError):
        OracleCase(Config(16, 48))  # jtot must be a power of two
    with pytest.raises(ValueError):
        OracleCase(Config(1, 32))
