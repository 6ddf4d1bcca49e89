"""TEST INFRASTRUCTURE ONLY -- build recipe for the CPU oracle.

* ``build/liboracle.so`` (the C restatement) is built everywhere.
* ``_ref/libsnsref.so`` (the reference's own sources + stand-ins) is built only
  when the reference source tree is present (``SNS_REFERENCE_DIR``, default
  ``/root/reference``); it is not needed by any GPU-side test.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DEFAULT = "/root/reference"


def _make(target: str, extra: list[str]) -> subprocess.CompletedProcess:
    return subprocess.run(["make", "-C", HERE, "-j8", target] + extra, capture_output=True, text=True)


def build(verbose: bool = False) -> dict:
    out = {}
    r = _make("liboracle", [])
    if r.returncode != 0:  # toolchains without OpenMP: the oracle is then single-threaded
        r = _make("liboracle", ["OMPFLAG="])
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    out["liboracle"] = os.path.join(HERE, "build", "liboracle.so")
    ref = os.environ.get("SNS_REFERENCE_DIR", REF_DEFAULT)
    if os.path.isfile(os.path.join(ref, "src", "fluid", "compute_potential.c")):
        r = _make("ref", [f"REF={ref}"])
        if r.returncode != 0:
            raise RuntimeError("reference build failed:\n" + r.stdout + r.stderr)
        out["libsnsref"] = os.path.join(HERE, "_ref", "libsnsref.so")
    if verbose:
        print(out)
    return out


if __name__ == "__main__":
    build(verbose=True)
