"""The batched FP32-stencil / FP64-Poisson form on the GPU.

Accuracy is measured against the FP64 CPU oracle (bit-identical to the
reference) run with the same dt and the explicit scheme, as relative L2 error
per field over the interior; the tolerances below are the stated bars of this
form. Batching must not change any case: a case computed alone and the same
case computed in a mix of other cases (admitted or retired mid-run) agree
bit for bit, because every case's arithmetic only reads its own data.
"""
import numpy as np
import pytest

from oracle.bindings import Config, OracleCase

pytestmark = pytest.mark.gpu

EXPLICIT_ONLY = [1.0, 1e30, 1e30, 1e30]  # cost table that always selects EXP(x)-EXP(y)
FIELDS = ("ux", "uy", "p", "temp")


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from simplenavierstokessolver_gb300.build import build

    build()


def interior(k, a):
    return a[1:-1, 1:-1] if k != "ux" else a[1:-1, 1:-1]


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def errors(got, ref):
    """relative L2 per field; p is compared modulo its mean: the pressure
    gauge (the null space of the Neumann Poisson problem) is pinned here,
    while on non-uniform grids the reference's zero-mode pivot is round-off
    rather than exactly zero and sets an arbitrary constant"""
    out = {}
    for k in FIELDS:
        a, b = interior(k, got[k]), interior(k, ref[k])
        if k == "p":
            a, b = a - a.mean(), b - b.mean()
        out[k] = rel_l2(a, b)
    return out


def oracle_fixed_dt(desc, steps, dt):
    from simplenavierstokessolver_gb300.batch import initial_temperature

    cfg = Config(desc.itot, desc.jtot, ly=desc.ly, stretch=desc.stretch, Ra=desc.Ra, Pr=desc.Pr)
    o = OracleCase(cfg, threads=4)
    st = o.get_state()
    o.set_state(st["ux"], st["uy"], st["p"], initial_temperature(desc))
    o.set_dt(dt, 0, 0)
    o.run(steps, decide=False)
    return o


def explicit_dt(desc):
    """the reference's first dt for this case with both directions explicit"""
    o = OracleCase(Config(desc.itot, desc.jtot, ly=desc.ly, stretch=desc.stretch, Ra=desc.Ra, Pr=desc.Pr))
    o.set_costs(EXPLICIT_ONLY)
    o.decide_dt()
    return o.get_dt()["dt"]


@pytest.mark.parametrize("stretch", [1e9, 3], ids=["uniform", "stretched"])
def test_single_case_matches_fp64_oracle(stretch):
    from simplenavierstokessolver_gb300.batch import Batch, Desc

    desc = Desc(64, 128, ly=2.0, stretch=stretch, Ra=1e6, Pr=1.0, seed=7)
    dt = explicit_dt(desc)
    desc.fixed_dt = dt
    with Batch(256 << 20) as b:
        s = b.add(desc)
        b.step(60)
        got = b.state(s)
        st = b.status(s)
    assert st["step"] == 60 and abs(st["time"] - 60 * dt) < 1e-12
    o = oracle_fixed_dt(desc, 60, dt)
    err = errors(got, o.get_state())
    assert max(err.values()) < 1e-5, err


@pytest.mark.parametrize("stretch", [1e9, 3], ids=["uniform", "stretched"])
def test_compensated_case_matches_fp64_oracle(stretch):
    """float-float stencil terms and increments: the error against the FP64
    oracle drops by orders of magnitude below the FP32 case's"""
    from simplenavierstokessolver_gb300.batch import Batch, Desc

    errs = {}
    for comp in (False, True):
        desc = Desc(64, 128, ly=2.0, stretch=stretch, Ra=1e6, Pr=1.0, seed=7, compensated=comp)
        dt = explicit_dt(desc)
        desc.fixed_dt = dt
        with Batch(256 << 20) as b:
            s = b.add(desc)
            b.step(60)
            got = b.state(s)
        errs[comp] = errors(got, oracle_fixed_dt(desc, 60, dt).get_state())
    assert max(errs[True].values()) < 1e-10, errs
    assert max(errs[True].values()) < 1e-3 * max(errs[False].values()), errs


def test_compensated_alone_and_next_to_fp32_cases_are_identical():
    """compensated cases run in a launch of their own over the tail of the
    tile list: mixing them with FP32 cases changes no case"""
    from simplenavierstokessolver_gb300.batch import Batch, Desc

    descs = [Desc(64, 128, Ra=3e6, Pr=0.7, seed=1, compensated=True), Desc(128, 256, Ra=1e8, Pr=5.0, seed=2),
             Desc(96, 64, ly=0.5, Ra=1e5, Pr=2.0, seed=3, stretch=4, compensated=True)]
    alone = []
    for d in descs:
        with Batch(512 << 20) as b:
            s = b.add(d)
            b.step(20)
            alone.append(b.state(s))
    with Batch(1 << 30) as b:
        slots = [b.add(d) for d in descs]
        b.step(20)
        mixed = [b.state(s) for s in slots]
    for a, m in zip(alone, mixed):
        for k in a:
            assert np.array_equal(a[k], m[k]), k


def test_cfl_dt_tracks_the_oracle():
    """dt from the device max-|u| reduction follows the reference's rule."""
    from simplenavierstokessolver_gb300.batch import Batch, Desc, initial_temperature

    desc = Desc(128, 256, ly=2.0, Ra=1e7, Pr=1.0, seed=3)
    cfg = Config(128, 256, ly=2.0, Ra=1e7, Pr=1.0)
    o = OracleCase(cfg, threads=4)
    st0 = o.get_state()
    o.set_state(st0["ux"], st0["uy"], st0["p"], initial_temperature(desc))
    o.set_costs(EXPLICIT_ONLY)
    with Batch(256 << 20) as b:
        s = b.add(desc)
        for n in (1, 20, 40):
            b.step(n)
            o.run(n)
            st = b.status(s)
            odt = o.get_dt()
            assert st["step"] == odt["step"]
            assert abs(st["time"] - odt["time"]) <= 1e-5 * odt["time"]
        err = errors(b.state(s), o.get_state())
    assert max(err.values()) < 1e-4, err


def test_projection_is_solenoidal():
    from simplenavierstokessolver_gb300.batch import Batch, Desc

    desc = Desc(256, 512, Ra=1e8, Pr=1.0, seed=11)
    with Batch(512 << 20) as b:
        s = b.add(desc)
        b.step(30)
        got = b.state(s)
    nx, ny = desc.itot, desc.jtot
    dx, dy = 1.0 / nx, 2.0 / ny
    ux, uy = got["ux"], got["uy"]
    div = (ux[1:-1, 1:] - ux[1:-1, :-1]) / dx + (uy[2:, 1:-1] - uy[1:-1, 1:-1]) / dy
    scale = max(np.abs(ux).max() / dx, np.abs(uy).max() / dy)
    assert np.abs(div).max() < 1e-5 * scale  # FP32 velocity: round-off level


def test_alone_and_in_the_mix_are_identical():
    from simplenavierstokessolver_gb300.batch import Batch, Desc

    descs = [Desc(64, 128, Ra=3e6, Pr=0.7, seed=1), Desc(128, 256, Ra=1e8, Pr=5.0, seed=2),
             Desc(96, 64, ly=0.5, Ra=1e5, Pr=2.0, seed=3, stretch=4), Desc(256, 512, Ra=1e9, Pr=1.0, seed=4)]
    alone = []
    for d in descs:
        with Batch(512 << 20) as b:
            s = b.add(d)
            b.step(25)
            alone.append(b.state(s))
    with Batch(1 << 30) as b:
        slots = [b.add(d) for d in descs]
        b.step(25)
        mixed = [b.state(s) for s in slots]
    for a, m in zip(alone, mixed):
        for k in a:
            assert np.array_equal(a[k], m[k]), k


def test_admission_retirement_and_completion():
    from simplenavierstokessolver_gb300 import _native as N
    from simplenavierstokessolver_gb300.batch import Batch, Desc, case_bytes

    small = Desc(64, 128, Ra=1e6, Pr=1.0, seed=21, steps=30)
    other = Desc(128, 256, Ra=1e7, Pr=1.0, seed=22)
    need = case_bytes(small) + case_bytes(other)
    with Batch(need + case_bytes(small) // 2) as b:  # room for exactly these two
        s1 = b.add(small)
        b.step(10)
        s2 = b.add(other)  # joins mid-run
        assert b.try_add(Desc(64, 128, seed=23)) is None  # does not fit: rejected, nothing changes
        b.step(40)  # small completes after its 30th step
        st = b.status(s1)
        assert st["done"] and st["step"] == 30
        got_small = b.state(s1)
        b.remove(s1)  # retire: memory returns to the arena
        s3 = b.add(Desc(64, 128, Ra=1e6, Pr=1.0, seed=24))
        b.step(5)
        assert b.status(s2)["step"] == 45 and b.status(s3)["step"] == 5
        got_other = b.state(s2)
    with Batch(256 << 20) as b:
        s = b.add(small)
        b.step(35)
        assert b.status(s)["step"] == 30
        ref_small = b.state(s)
    with Batch(256 << 20) as b:
        s = b.add(other)
        b.step(45)
        ref_other = b.state(s)
    for k in ref_small:
        assert np.array_equal(got_small[k], ref_small[k]), k
        assert np.array_equal(got_other[k], ref_other[k]), k
    assert N.SNS_ERR_OOM == 4


def test_unsupported_sizes_are_rejected():
    from simplenavierstokessolver_gb300 import _native as N
    from simplenavierstokessolver_gb300.batch import Batch, Desc

    with Batch(64 << 20) as b:
        for d in (Desc(48, 64), Desc(64, 96), Desc(64, 4)):
            with pytest.raises(N.SnsError):
                b.add(d)


def test_serving_results_equal_standalone_runs():
    """Continuous batching: requests arriving while others run are admitted
    when arena memory frees up; every request's final state equals the same
    case run alone."""
    from simplenavierstokessolver_gb300.batch import Batch, Desc, case_bytes, serve

    # every other request compensated: both kinds share the launches
    descs = [Desc(64, 128, Ra=1e6 * (k + 1), Pr=1.0 + 0.3 * k, seed=100 + k, steps=20 + 7 * k, compensated=k % 2 == 1)
             for k in range(5)]
    descs.append(Desc(128, 256, Ra=1e8, Pr=0.8, seed=200, steps=25))
    arrivals = [0.0, 0.0, 0.05, 0.1, 0.1, 0.15]
    arena = case_bytes(descs[-1]) + case_bytes(descs[0])  # at most ~2 cases resident
    r = serve(descs, arrivals, hbm_bytes=arena, max_cases=8, chunk_steps=5, keep_states=True)
    assert len(r["states"]) == len(descs)
    assert all(r["done"][k] >= r["admit"][k] >= arrivals[k] for k in range(len(descs)))
    for k, d in enumerate(descs):
        with Batch(case_bytes(d) + (1 << 20)) as b:
            s = b.add(d)
            b.step(d.steps + 3)  # finished cases stop at their step count
            alone = b.state(s)
        for f in alone:
            assert np.array_equal(alone[f], r["states"][k][f]), (k, f)


def test_batch_diagnostics_match_host_evaluation():
    """sns_batch_diagnostics against the oracle's log quantities evaluated on
    the batch's own (FP32) state"""
    from simplenavierstokessolver_gb300.batch import Batch, Desc

    d = Desc(64, 128, Ra=1e7, Pr=1.0, seed=9)
    with Batch(256 << 20) as b:
        s = b.add(d)
        b.step(25)
        dg = b.diagnostics(s)
        st = b.state(s)
    o = OracleCase(Config(64, 128, Ra=1e7, Pr=1.0))
    o.set_state(st["ux"], st["uy"], st["p"], st["temp"])
    dr = o.diagnostics()
    scale = np.maximum(np.abs(dr[1:]), 1e-12)
    assert np.all(np.abs(dg[1:] - dr[1:]) <= 1e-10 * scale + 1e-13), (dg, dr)
    assert abs(dg[0] - dr[0]) <= 1e-12 * dr[0]


def test_tuning_changes_speed_not_results():
    """every launch shape computes the same arithmetic per point: results are
    identical; the autotuner leaves the cases' state untouched"""
    from simplenavierstokessolver_gb300.batch import Batch, Desc

    descs = [Desc(64, 128, Ra=3e6, Pr=0.7, seed=1), Desc(128, 256, Ra=1e8, Pr=5.0, seed=2),
             Desc(96, 64, ly=0.5, Ra=1e5, Pr=2.0, seed=3, stretch=4)]
    shapes = [dict(tile_x=64, tile_rows=8, modes_per_block=4, fcols_shift=0),
              dict(tile_x=32, tile_rows=16, modes_per_block=8, fcols_shift=1),
              dict(tile_x=128, tile_rows=4, modes_per_block=2, fcols_shift=-1)]
    results = []
    for shape in shapes:
        with Batch(1 << 30) as b:
            slots = [b.add(d) for d in descs]
            b.set_tuning(**shape)
            b.step(12)
            results.append([b.state(s) for s in slots])
    for other in results[1:]:
        for a, m in zip(results[0], other):
            for k in a:
                assert np.array_equal(a[k], m[k]), k
    with Batch(1 << 30) as b:
        slots = [b.add(d) for d in descs]
        b.step(5)
        before = [b.state(s) for s in slots]
        st_before = [b.status(s) for s in slots]
        chosen, ms = b.autotune(steps=3)
        assert ms > 0 and chosen["tile_x"] in (32, 64, 128)
        after = [b.state(s) for s in slots]
        assert [b.status(s) for s in slots] == st_before
        for a, m in zip(before, after):
            for k in a:
                assert np.array_equal(a[k], m[k]), k
        b.step(7)  # continuing with the tuned shapes gives the untuned run's results
        tuned = [b.state(s) for s in slots]
    for a, m in zip(results[0], tuned):
        for k in a:
            assert np.array_equal(a[k], m[k]), k


@pytest.mark.parametrize("compensated", [False, True], ids=["fp32", "compensated"])
def test_checkpoint_and_restart_continue_bit_for_bit(tmp_path, compensated):
    """serving snapshot and resume: a case checkpointed after 15 steps and
    admitted from the files into another batch continues as the uninterrupted
    case; the files read back as the reference's save layout. An FP32 case
    continues bit for bit (its pairs carry the increments' FP32 precision and
    fit the file's FP64 values); a compensated pair can hold more bits than
    an FP64 value, so that case resumes from the pair rounded to FP64"""
    from simplenavierstokessolver_gb300.batch import Batch, Desc

    d = Desc(128, 256, Ra=1e8, Pr=1.0, seed=5, compensated=compensated)
    with Batch(512 << 20) as b:
        s = b.add(d)
        b.step(15)
        b.checkpoint(s, str(tmp_path / "ck"))
        b.step(10)
        straight = b.state(s)
        st_straight = b.status(s)
    assert int(np.load(tmp_path / "ck" / "step.npy")) == 15
    assert np.load(tmp_path / "ck" / "ux.npy").shape == (256, 129)
    with Batch(512 << 20) as b:
        s = b.add_restart(d, str(tmp_path / "ck"))
        assert b.status(s)["step"] == 15
        b.step(10)
        resumed = b.state(s)
        st_resumed = b.status(s)
    assert st_resumed["step"] == st_straight["step"] and st_resumed["time"] == st_straight["time"]
    for k in ("ux", "uy", "p", "temp"):
        if compensated:
            a, r = resumed[k][1:-1, 1:-1], straight[k][1:-1, 1:-1]
            assert np.linalg.norm(a - r) <= 1e-13 * np.linalg.norm(r), k
        else:
            assert np.array_equal(straight[k], resumed[k]), k


def test_restart_from_a_plain_checkpoint(tmp_path):
    """a plain-path checkpoint (the reference's save layout, byte-identical to
    its save() files) admits into a batch: the FP64 state is held exactly up
    to the compensated pairs' ~48 significant bits"""
    from simplenavierstokessolver_gb300.batch import Batch, Desc
    from simplenavierstokessolver_gb300.solver import Case

    with Case(64, 128, Ra=1e7, Pr=1.0) as c:
        c.run(20)
        c.checkpoint(str(tmp_path / "plain"))
        c.checkpoint_wait()
        ref = c.get_state()
    with Batch(256 << 20) as b:
        s = b.add_restart(Desc(64, 128, Ra=1e7, Pr=1.0), str(tmp_path / "plain"))
        got = b.state(s)
        assert b.status(s)["step"] == 20
    for k in ("ux", "uy", "temp"):  # FP64 values held as compensated FP32 pairs: ~2^-48 relative
        assert np.abs(got[k] - ref[k])[1:-1, 1:-1].max() <= 1e-13 * max(np.abs(ref[k]).max(), 1.0), k
    assert np.array_equal(got["p"][1:-1, 1:-1], ref["p"][1:-1, 1:-1])


@pytest.mark.parametrize("shape", [dict(tile_x=64, tile_rows=8, modes_per_block=4, fcols_shift=0),
                                   dict(tile_x=128, tile_rows=4, modes_per_block=2, fcols_shift=-1)],
                         ids=["64x8_mpb4", "128x4_mpb2"])
def test_persistent_substage_launch_matches_the_per_phase_launches(shape):
    """one persistent cooperative launch per substage (its blocks walk every
    phase's work list, a grid barrier between phases) against the graph of
    per-phase launches: the same device functions per work item; the batched
    unit is compiled with contraction and the compiler may pair multiply-adds
    differently in the two kernels, so the FP32 cases agree to their rounding
    (a work item skipped or done twice would be off by O(1)), compensated
    cases far closer"""
    from simplenavierstokessolver_gb300.batch import Batch, Desc

    descs = [Desc(64, 128, Ra=3e6, Pr=0.7, seed=1), Desc(128, 256, Ra=1e8, Pr=5.0, seed=2),
             Desc(96, 64, ly=0.5, Ra=1e5, Pr=2.0, seed=3, stretch=4),
             Desc(64, 64, ly=1.0, Ra=1e6, Pr=1.0, seed=4, compensated=True)]
    results = []
    for persistent in (False, True):
        with Batch(1 << 30) as b:
            slots = [b.add(d) for d in descs]
            b.set_tuning(**shape)
            b.set_persistent(persistent)
            b.step(9)
            b.synchronize()
            results.append([b.state(s) for s in slots])
            if persistent:
                b.set_persistent(False)  # and back: the per-phase form continues
                b.step(1)
                b.synchronize()
    for d, a, m in zip(descs, results[0], results[1]):
        bar = 1e-9 if d.compensated else 1e-5
        for k in ("ux", "uy", "temp", "p"):
            r = a[k][1:-1, 1:-1] - (a[k][1:-1, 1:-1].mean() if k == "p" else 0.0)
            g = m[k][1:-1, 1:-1] - (m[k][1:-1, 1:-1].mean() if k == "p" else 0.0)
            err = np.linalg.norm(g - r) / np.linalg.norm(r)
            assert err <= bar, (d, k, err)
