"""Recipe: build the reference's own segmentation code for the CPU.

Test infrastructure only.  Compiles nitronoid/split's hot-path sources
(k-means, connected components, label compression, small-segment merge,
erosion, Sobel normals) with g++ against CUDA 13's Thrust using the OpenMP
device system, through the CUSP container subset in oracle/cusp_shim, and
links them with oracle/ref_driver.cpp into oracle/_ref/libsplitref.so.

The reference sources are read from REF_ROOT (the SPLIT_REF_ROOT environment
variable, else /root/reference, where this recipe's build machine mounts the
reference read-only) and copied into the git-ignored oracle/_ref/src, where two mechanical edits are
applied to the copies (the reference itself is never modified and nothing of
it is committed):
  1. member ``x.get<N>()`` becomes ``thrust::get<N>(x)``: CCCL 3's
     thrust::tuple is cuda::std::tuple, which has no member get;
  2. oracle/ref_prelude.h is force-included (host min/max, stand-ins that let
     g++ parse the one never-launched kernel);
  3. merge_smooth_boundaries.cu:216-226 gets thrust::minimum instead of the
     predicate thrust::less as its reduction (PATCHES below): as written the
     file does not compile, and its comment says it takes the smallest value.
When the copied sources are present but the reference is not (another
machine), the copies are compiled as they are.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _reference_root() -> str:
    """SPLIT_REF_ROOT, else the read-only mount /root/reference if present; ""
    otherwise (the staged copies are then compiled as they are)."""
    env = os.environ.get("SPLIT_REF_ROOT")
    if env:
        return env
    return "/root/reference" if os.path.isdir("/root/reference") else ""


REF_ROOT = _reference_root()
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "src")
BUILD = os.path.join(OUT, "build", platform.machine())
LIB = os.path.join(BUILD, "libsplitref.so")

SOURCES = [
    "split/src/split/device/kmeans/cluster.cu",
    "split/src/split/device/kmeans/label.cu",
    "split/src/split/device/kmeans/centroids.cu",
    "split/src/split/device/kmeans/propagation.cu",
    "split/src/split/device/ccl/connected_components.cu",
    "split/src/split/device/ccl/compress_labels.cu",
    "split/src/split/device/ccl/segment_adjacency.cu",
    "split/src/split/device/ccl/merge_small_segments.cu",
    "split/src/split/device/morph/erode.cu",
    "split/src/split/device/sfs/sobel_normals.cu",
    "split/src/split/device/detail/normalize_vectors.cu",
    "split/src/split/device/color/beta_feature.cu",
    "split/src/split/device/ccl/merge_smooth_boundaries.cu",
]

# Headers a source used through includes of the Thrust / CUSP versions it was
# written against (added to that file's staged copy only).
EXTRA_INCLUDES = {"beta_feature.cu": ("thrust/extrema.h",)}

# One-token fixes without which a source does not compile, applied to its
# staged copy only:
#   merge_smooth_boundaries.cu:216-226 hands reduce_by_key the predicate
#   thrust::less as its reduction ("If we are faced with multiple options, we
#   take the smallest scalar"); the functor that takes the smaller value is
#   thrust::minimum, which is what the comment describes.
PATCHES = {"merge_smooth_boundaries.cu": (("thrust::less<thrust::tuple<real, int>>()",
                                           "thrust::minimum<thrust::tuple<real, int>>()"),)}

_GET = re.compile(r"\.get<(\d+)>\(\)")
_IDENT = re.compile(r"[A-Za-z0-9_]")


def _receiver_start(s: str, end: int) -> int:
    """Start index of the postfix expression ending just before `end`."""
    i = end
    while True:
        # trailing call / subscript groups
        while i > 0 and s[i - 1] in ")]":
            close = s[i - 1]
            open_ = "(" if close == ")" else "["
            depth = 0
            j = i - 1
            while j >= 0:
                if s[j] == close:
                    depth += 1
                elif s[j] == open_:
                    depth -= 1
                    if depth == 0:
                        break
                j -= 1
            i = j
        # template argument list directly before (e.g. get<0>)
        if i > 0 and s[i - 1] == ">":
            depth = 0
            j = i - 1
            while j >= 0:
                if s[j] == ">":
                    depth += 1
                elif s[j] == "<":
                    depth -= 1
                    if depth == 0:
                        break
                j -= 1
            i = j
        while i > 0 and _IDENT.match(s[i - 1]):
            i -= 1
        if i >= 2 and s[i - 2:i] == "::":
            i -= 2
            continue
        if i >= 1 and s[i - 1] == "." and not (i >= 2 and s[i - 2].isdigit()):
            i -= 1
            continue
        if i >= 2 and s[i - 2:i] == "->":
            i -= 2
            continue
        return i


def rewrite_get(text: str) -> str:
    """Rewrite every member ``.get<N>()`` to ``thrust::get<N>(receiver)``."""
    while True:
        m = _GET.search(text)
        if not m:
            return text
        start = _receiver_start(text, m.start())
        recv = text[start:m.start()]
        text = text[:start] + f"thrust::get<{m.group(1)}>({recv})" + text[m.end():]


def stage_sources(verbose: bool = False) -> bool:
    """Copy + patch the reference sources into oracle/_ref/src.  Returns False
    when neither the reference nor an earlier copy is available."""
    ref_split = os.path.join(REF_ROOT, "split") if REF_ROOT else ""
    if not ref_split or not os.path.isdir(ref_split):
        return os.path.isdir(os.path.join(SRC, "include"))
    if os.path.isdir(SRC):
        shutil.rmtree(SRC)
    os.makedirs(SRC)
    shutil.copytree(os.path.join(ref_split, "include"), os.path.join(SRC, "include"))
    for rel in SOURCES:
        dst = os.path.join(SRC, os.path.basename(rel)[:-3] + ".cpp")
        with open(os.path.join(REF_ROOT, rel)) as f:
            text = f.read()
        extra = "".join(f"#include <{h}>\n" for h in EXTRA_INCLUDES.get(os.path.basename(rel), ()))
        for old, new in PATCHES.get(os.path.basename(rel), ()):
            if text.count(old) != 1:
                raise RuntimeError(f"{rel}: the patched expression is not there once")
            text = text.replace(old, new)
        with open(dst, "w") as f:
            f.write(extra + rewrite_get(text))
    for root, _, files in os.walk(os.path.join(SRC, "include")):
        for name in files:
            p = os.path.join(root, name)
            with open(p) as f:
                text = f.read()
            new = rewrite_get(text)
            if new != text:
                with open(p, "w") as f:
                    f.write(new)
    if verbose:
        print(f"staged reference sources in {SRC}")
    return True


def _cxx_flags() -> list[str]:
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    return ["-O2", "-std=c++17", "-fPIC", "-fopenmp", "-w",
            "-DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_OMP",
            "-DTHRUST_HOST_SYSTEM=THRUST_HOST_SYSTEM_CPP",
            "-include", os.path.join(HERE, "ref_prelude.h"),
            "-I", os.path.join(HERE, "cusp_shim"), "-I", os.path.join(SRC, "include"),
            "-I", os.path.join(cuda_inc, "cccl"), "-I", cuda_inc]


def _compile(args):
    src, obj = args
    r = subprocess.run(["g++", *_cxx_flags(), "-c", "-o", obj, src], capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f"g++ failed on {os.path.basename(src)}:\n{r.stderr[-4000:]}")
    return obj


def build(verbose: bool = False, force: bool = False) -> str | None:
    """Build oracle/_ref/build/<machine>/libsplitref.so; None when the
    reference sources are unavailable."""
    if not stage_sources(verbose) and not os.path.exists(LIB):
        if verbose:
            print("reference sources unavailable: CPU reference not built")
        return None
    if os.path.exists(LIB) and not force:
        newest = max(os.path.getmtime(os.path.join(r, f)) for r, _, fs in os.walk(SRC) for f in fs)
        if os.path.getmtime(LIB) >= max(newest, os.path.getmtime(os.path.join(HERE, "ref_driver.cpp"))):
            return LIB
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith(".cpp"))
    srcs.append(os.path.join(HERE, "ref_driver.cpp"))
    jobs = [(s, os.path.join(BUILD, os.path.basename(s)[:-4] + ".o")) for s in srcs]
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, jobs))
    r = subprocess.run(["g++", "-shared", "-fopenmp", "-o", LIB, *objs], capture_output=True,
                       text=True)
    if r.returncode:
        raise RuntimeError("link failed:\n" + r.stderr[-4000:])
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
