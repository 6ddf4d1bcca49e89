"""NPY format of checkpoints against the files the reference's own save()
wrote (tests/golden/save_rb_uniform_32x64, made by make_golden.py): the
library's writer reproduces them byte for byte and its reader loads them.
Host code only: no device is needed."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "save_rb_uniform_32x64")
SCALARS = {"step": np.int32, "itot": np.int32, "jtot": np.int32, "time": np.float64, "lx": np.float64,
           "ly": np.float64, "Ra": np.float64, "Pr": np.float64}


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from simplenavierstokessolver_gb300.build import build

    build()


def names():
    return sorted(f[:-4] for f in os.listdir(GOLD) if f.endswith(".npy"))


@pytest.mark.parametrize("name", names())
def test_writer_reproduces_the_reference_files(tmp_path, name):
    from simplenavierstokessolver_gb300.solver import npy_read, npy_write

    ref = np.load(os.path.join(GOLD, name + ".npy"))
    dtype = SCALARS.get(name, np.float64)
    got = npy_read(os.path.join(GOLD, name + ".npy"), ref.shape, dtype)
    assert np.array_equal(got, ref)
    out = tmp_path / (name + ".npy")
    npy_write(str(out), got)
    with open(os.path.join(GOLD, name + ".npy"), "rb") as a, open(out, "rb") as b:
        assert a.read() == b.read()


def test_reader_accepts_numpy_files_and_checks_shapes(tmp_path):
    from simplenavierstokessolver_gb300 import _native as N
    from simplenavierstokessolver_gb300.solver import npy_read

    a = np.arange(12.0).reshape(3, 4)
    np.save(tmp_path / "a.npy", a)
    assert np.array_equal(npy_read(str(tmp_path / "a.npy"), (3, 4)), a)
    with pytest.raises(N.SnsError, match="shape"):
        npy_read(str(tmp_path / "a.npy"), (4, 3))
    with pytest.raises(N.SnsError, match="dtype"):
        npy_read(str(tmp_path / "a.npy"), (3, 4), np.int32)
    with pytest.raises(N.SnsError, match="cannot open"):
        npy_read(str(tmp_path / "missing.npy"), (3, 4))
