"""Build recipe for libsns_gpu.so (sm_103a only), in-tree.

Each translation unit is compiled in parallel; host code and the FP64 kernels
are compiled without floating-point contraction so that the plain path keeps
the reference's rounding. Objects go to ``_build/``, the library to
``_lib/libsns_gpu.so``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libsns_gpu.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> str:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


# translation unit -> extra flags. fmad=false: bit-identical FP64 path.
UNITS = {
    "plain_fp64.cu": ["--fmad=false"],
    # the same kernels with contraction (the parallel form)
    "plain_fp64_contract.cu": ["--fmad=true"],
    "batch_fp32.cu": [],
    "diagnostics.cu": [],
    "fp64_rate.cu": [],
    "plain_parallel.cu": [],
    "sns_api.cpp": [],
    "batch_api.cpp": [],
    "npy.cpp": [],
    "cost_model.cpp": [],
}


# units that include another unit's source
INCLUDES = {"plain_fp64_contract.cu": ["plain_fp64.cu"]}


def _headers():
    hs = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh", ".inc"))]
    return hs


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(unit: str, extra: list[str], cuda: str) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD, unit + ".o")
    # a unit that includes another .cu rebuilds with it
    deps = [src, __file__] + _headers() + [os.path.join(CSRC, u) for u in INCLUDES.get(unit, [])]
    if not _stale(obj, deps):
        return obj
    nvcc = os.path.join(cuda, "bin", "nvcc")
    if unit.endswith(".cu"):
        cmd = [nvcc, "-c", src, "-o", obj, "-O3", "-std=c++17", "-lineinfo", *ARCH, "-Xptxas", "-v",
               "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I", INCLUDE, "-I", CSRC, *extra]
    else:
        cmd = ["g++", "-c", src, "-o", obj, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off",
               "-I", INCLUDE, "-I", CSRC, "-I", os.path.join(cuda, "include"), *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compiling {unit} failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    with open(obj + ".log", "w") as fh:
        fh.write(r.stdout + r.stderr)
    return obj


def build(verbose: bool = False) -> str:
    cuda = cuda_home()
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], cuda), UNITS.items()))
    if _stale(LIB, objs):
        cmd = [os.path.join(cuda, "bin", "nvcc"), "-shared", *ARCH, "-o", LIB, *objs,
               "-L", os.path.join(cuda, "lib64"), "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"linking failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
