"""Build libps_b200.so (the GB300 stencil library) in-tree with nvcc for sm_103a.

    python parallelstencil.jl_gb300/build.py [--force] [--jobs N]
    (or ``from ps_gb300._build import build; build()``)

Each ``csrc/*.cu`` is compiled to an object in ``_build/`` (in parallel), then linked into
``parallelstencil.jl_gb300/lib/libps_b200.so`` with the CUDA runtime linked statically, so the
library loads on a machine without a GPU driver (its symbols can be inspected there) and
reaches the driver lazily at ``ps_init``. All kernels are built with ``--fmad=false``: the
reference (Julia) never contracts ``a*b+c`` into an FMA, and bit-identical FP64 results need
the same rounding.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))  # parallelstencil.jl_gb300/
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libps_b200.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC,-O2",
                     "-I", INCLUDE, "-I", CSRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + [os.path.join(INCLUDE, "ps_gb300.h")]


def _compile(src: str, force: bool) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    newest = max([os.path.getmtime(src)] + [os.path.getmtime(d) for d in _deps()])
    if not force and os.path.exists(obj) and os.path.getmtime(obj) >= newest:
        return obj
    cmd = [nvcc()] + NVCC_FLAGS + ["-c", src, "-o", obj + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    os.replace(obj + ".tmp", obj)
    return obj


def build(force: bool = False, jobs: int | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, force), srcs))
    newest = max(os.path.getmtime(o) for o in objs)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        tmp = LIB + ".tmp%d" % os.getpid()
        # NVRTC (run-time compilation of @parallel kernel bodies) from the toolkit the library is built with
        root = os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))
        cands = [os.path.join(root, d) for d in ("lib64", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib", "lib")]
        cudalib = next((d for d in cands if os.path.exists(os.path.join(d, "libnvrtc.so"))), cands[0])
        cmd = [nvcc()] + ARCH + ["-shared", "-Xcompiler", "-fPIC", "-o", tmp] + objs + \
            ["-L" + cudalib, "-lnvrtc", "-Xlinker", "-rpath", "-Xlinker", cudalib]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--jobs", type=int, default=None)
    a = ap.parse_args(argv)
    print(build(force=a.force, jobs=a.jobs))
    return 0


if __name__ == "__main__":
    sys.exit(main())
