"""The partition method's host factors (csrc/host_common.h,
partition_factors_tri), checked on the CPU: tests/c/partition_check.cpp
applies the GPU kernels' operations (interior elimination and substitution
per segment, interface right-hand sides, PCR over the 32 interface unknowns
with cyclic lane indices, spikes) to random diagonally dominant lines,
wall-bounded and periodic, with constant and varying coefficients, 64 to
512 rows (odd segment lengths included), and compares each solution with a
dense Gaussian elimination of the same system. The same program with the
periodic wrap-around couplings dropped from the solve must fail the
comparison: the check sees a wrong coupling.
"""
import pathlib
import shutil
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = tmp_path_factory.mktemp("partition") / "partition_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(ROOT / "simplenavierstokessolver_gb300" / "csrc"),
                    str(ROOT / "tests" / "c" / "partition_check.cpp"), "-o", str(exe)], check=True)
    return exe


def _run(exe, *args):
    out = subprocess.run([str(exe), *args], check=True, capture_output=True, text=True).stdout
    return [(int(n), int(p), int(c), float(e)) for n, p, c, e in (line.split() for line in out.splitlines())]


def test_partition_solve_matches_dense_solve(checker):
    rows = _run(checker)
    assert len(rows) == 20
    for n, periodic, constant, err in rows:
        assert err < 1e-14, (n, periodic, constant, err)


def test_dropped_wraparound_is_detected(checker):
    rows = _run(checker, "nowrap")
    periodic = [err for n, p, c, err in rows if p]
    walls = [err for n, p, c, err in rows if not p]
    assert min(periodic) > 1e-3
    assert max(walls) < 1e-14
