"""Build libaqua.so in-tree for sm_103a.

Translation units compile in parallel (g++ for host-only C++, nvcc for CUDA),
objects go to ``_build/`` beside this file, and the shared library is linked
with the CUDA runtime statically so that it loads without a toolkit on the
library path. Run ``python build.py`` or call ``build()``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libaqua.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _sources():
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    return cpp, cu


def _newer(src_paths, target) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(p) > t for p in src_paths)


def build(verbose: bool = False, force: bool = False) -> str:
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OUT_DIR, exist_ok=True)
    cpp, cu = _sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "aqua.h"))
    inc = ["-I" + CSRC, "-I" + os.path.join(HERE, "..", "include"), "-I" + os.path.join(cuda, "include")]
    host_flags = ["-O3", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off", "-Wall",
                  "-Wno-unused-function"]
    jobs = []
    objs = []
    for f in cpp:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT_DIR, f + ".o")
        objs.append(obj)
        if force or _newer([src] + headers, obj):
            jobs.append(["g++", *host_flags, *inc, "-c", src, "-o", obj])
    for f in cu:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT_DIR, f + ".o")
        objs.append(obj)
        if force or _newer([src] + headers, obj):
            jobs.append([nvcc, ARCH, "-lineinfo", "-O3", "-std=c++17", "--expt-relaxed-constexpr",
                         "-Xcompiler", "-fPIC,-fvisibility=hidden,-ffp-contract=off", *inc,
                         "-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, flush=True)

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    if force or jobs or _newer(objs, LIB):
        tmp = LIB + ".tmp"
        run([nvcc, ARCH, "-shared", "-o", tmp, *objs, "-lpthread"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
