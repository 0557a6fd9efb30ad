"""In-tree build of the native library (and the CPU oracle used by the tests).

libsplit_gb300.so: every CUDA translation unit under csrc/ compiled for
sm_103a only (``-gencode arch=compute_103a,code=sm_103a``), linked with the
static CUDA runtime.  Objects are compiled in parallel; a unit is rebuilt only
when it or a header is newer than its object.  (The seeded input generators
are a separate library, split_synth.)
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build", platform.machine())
STAMP = os.path.join(BUILD, "lib.stamp")
LIB = os.path.join(HERE, "libsplit_gb300.so")

ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_BUILD = os.path.join(ORACLE_DIR, "_build", platform.machine())
ORACLE_LIB = os.path.join(ORACLE_BUILD, "liboracle.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr", "-Xptxas", "-O3"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsplit_gb300")


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    inc = os.path.join(ROOT, "include")
    hs += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    return hs


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError(f"build step failed: {os.path.basename(cmd[-1])}")


def build_library(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = _headers()
    cus = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    steps = []
    objs = []
    for f in cus:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f[:-3] + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            steps.append([nvcc, *ARCH, *NVCC_FLAGS, "-c", "-o", obj, src])
    if steps:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
            list(ex.map(_run, steps))
    # the stamp lives in the per-machine build directory, so a library built
    # on another architecture is always relinked here
    if steps or _stale(STAMP, objs) or not os.path.exists(LIB):
        _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs, "-lm"])
        with open(STAMP, "w") as f:
            f.write(platform.machine() + "\n")
    if verbose:
        print(f"built {LIB}")
    return LIB


def build_oracle(verbose: bool = False) -> str:
    os.makedirs(ORACLE_BUILD, exist_ok=True)
    src = os.path.join(ORACLE_DIR, "oracle.c")
    if _stale(ORACLE_LIB, [src]):
        _run(["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off", "-fopenmp",
              "-o", ORACLE_LIB, src, "-lm"])
    if verbose:
        print(f"built {ORACLE_LIB}")
    return ORACLE_LIB


if __name__ == "__main__":
    build_library(verbose=True)
    build_oracle(verbose=True)
