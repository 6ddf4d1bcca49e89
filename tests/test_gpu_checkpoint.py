"""Checkpoint / restart of device-resident state in the reference's save
layout. The fused step equals the reference bit for bit, so after the golden
case's 25 steps the checkpoint files must equal, byte for byte, the files the
reference's own save() wrote (tests/golden/save_rb_uniform_32x64)."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(__file__)
GOLD = os.path.join(HERE, "golden", "save_rb_uniform_32x64")


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from simplenavierstokessolver_gb300.build import build

    build()


def golden_case():
    from simplenavierstokessolver_gb300.solver import Case

    with open(os.path.join(HERE, "golden", "manifest.json")) as fh:
        m = json.load(fh)["rb_uniform_32x64"]
    cfg = m["config"]
    c = Case(cfg["itot"], cfg["jtot"], ly=cfg["ly"], stretch=cfg["stretch"], Ra=cfg["Ra"], Pr=cfg["Pr"],
             costs=m["costs"])
    return c, m["steps"]


def same_files(d1, d2):
    n1 = sorted(os.listdir(d1))
    assert n1 == sorted(os.listdir(d2))
    for n in n1:
        with open(os.path.join(d1, n), "rb") as a, open(os.path.join(d2, n), "rb") as b:
            assert a.read() == b.read(), n


def test_checkpoint_equals_the_reference_save(tmp_path):
    c, steps = golden_case()
    with c:
        c.run(steps)
        c.checkpoint(str(tmp_path / "ck"))
        c.run(7)  # keeps stepping while the writer runs: the files hold the state at the call
        c.checkpoint_wait()
    same_files(tmp_path / "ck", GOLD)


def test_restart_continues_bit_for_bit(tmp_path):
    c, steps = golden_case()
    with c:
        c.run(steps + 10)
        straight = c.get_state()
        dt_straight = c.get_dt()
    r, _ = golden_case()
    with r:
        r.restart(GOLD)  # the reference's own files
        assert r.get_dt()["step"] == steps
        r.run(10)
        again = r.get_state()
        dt_again = r.get_dt()
    for k in ("ux", "uy", "p", "temp"):
        assert np.array_equal(straight[k], again[k]), k
    assert dt_again["time"] == dt_straight["time"] and dt_again["step"] == dt_straight["step"]


def test_restart_rejects_mismatched_files(tmp_path):
    from simplenavierstokessolver_gb300 import _native as N
    from simplenavierstokessolver_gb300.solver import Case

    with Case(64, 128) as c:
        with pytest.raises(N.SnsError, match="shape"):
            c.restart(GOLD)
        with pytest.raises(N.SnsError, match="cannot open"):
            c.restart(str(tmp_path / "nothing"))


def test_statistics_equal_the_reference_output(tmp_path):
    """statistics collected after every step of the golden case, written
    like statistics_output: byte for byte the reference's own files
    (tests/golden/stat_rb_uniform_32x64)."""
    from simplenavierstokessolver_gb300.solver import Statistics

    c, steps = golden_case()
    with c, Statistics(c) as st:
        for _ in range(steps):
            c.run(1)
            st.collect()
        assert st.num == steps
        st.output_to(str(tmp_path / "stat"))
    same_files(tmp_path / "stat", os.path.join(HERE, "golden", "stat_rb_uniform_32x64"))


def test_failed_checkpoint_is_reported_by_the_next_one(tmp_path):
    """a checkpoint whose writer fails (its directory cannot be created: a
    file stands in the path) is reported by the next sns_checkpoint, once;
    the call after that writes normally"""
    from simplenavierstokessolver_gb300 import SnsError

    blocker = tmp_path / "not_a_dir"
    blocker.write_text("a file where the checkpoint directory would go")
    c, steps = golden_case()
    with c:
        c.run(steps)
        c.checkpoint(str(blocker / "ck"))  # enqueued; the writer thread fails later
        with pytest.raises(SnsError):
            c.checkpoint(str(tmp_path / "good"))
        c.checkpoint(str(tmp_path / "good"))
        c.checkpoint_wait()
    same_files(tmp_path / "good", GOLD)
