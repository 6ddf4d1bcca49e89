"""The C ABI from a plain C99 program (tests/c/driver.c), as the reference's
own driver would call it: it must compile with -std=c99 -pedantic against
include/sns_gpu.h and link against libsns_gpu.so (CPU), and on a GPU it must
reproduce the reference's own result for the 32 x 64 golden case."""
import os
import platform
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    from simplenavierstokessolver_gb300.build import LIB, LIBDIR, build

    build()
    exe = str(tmp_path_factory.mktemp("c") / "driver")
    cmd = ["gcc", "-std=c99", "-pedantic", "-Wall", "-Wextra", "-Werror", "-O2", "-I", os.path.join(ROOT, "include"),
           os.path.join(HERE, "c", "driver.c"), "-o", exe, "-L", LIBDIR, "-lsns_gpu", f"-Wl,-rpath,{LIBDIR}"]
    subprocess.run(cmd, check=True)
    assert os.path.exists(LIB)
    return exe


def test_driver_compiles_and_links(driver):
    assert os.access(driver, os.X_OK)


@pytest.mark.gpu
def test_driver_reproduces_the_reference(driver, tmp_path):
    out = tmp_path / "state.bin"
    subprocess.run([driver, str(out)], check=True, timeout=300)
    nx, ny = 32, 64
    raw = np.fromfile(out, dtype=np.float64)
    su, sc = (ny + 2) * (nx + 1), (ny + 2) * (nx + 2)
    ux = raw[:su].reshape(ny + 2, nx + 1)
    uy = raw[su:su + sc].reshape(ny + 2, nx + 2)
    p = raw[su + sc:su + 2 * sc].reshape(ny + 2, nx + 2)
    t = raw[su + 2 * sc:su + 3 * sc].reshape(ny + 2, nx + 2)
    g = np.load(os.path.join(HERE, "golden", "rb_uniform_32x64.npz"))
    for name, a in (("ux", ux), ("uy", uy), ("p", p), ("temp", t)):
        ref = g[f"final_{name}"]
        if platform.machine() == "x86_64":
            assert np.array_equal(a, ref), name
        else:  # host libm of another architecture may differ in the last bit of the grid set-up
            assert np.linalg.norm(a - ref) <= 1e-12 * np.linalg.norm(ref), name
