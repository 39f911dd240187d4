"""Build recipe of the CPU oracle (test infrastructure): oracle.cpp ->
liboracle.so beside this file. -ffp-contract=off keeps one rounding per float
operation, which the bit-exact traversal comparison depends on.

The reference (`arukas`) has no compilable source for this path (src/lib.rs is
empty), so there is no oracle/_ref build.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")


def build(verbose: bool = False) -> str:
    src = os.path.join(HERE, "oracle.cpp")
    deps = [src, os.path.join(HERE, "oracle.h"), os.path.join(HERE, "..", "include", "aqua.h")]
    if os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-Wall",
           src, "-o", LIB + ".tmp"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
