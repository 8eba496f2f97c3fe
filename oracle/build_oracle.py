"""Build recipe for the parity oracle (test infrastructure, not the product).

Compiles oracle/*.cpp with g++ into oracle/_build/liboracle.so. The flags
matter for parity: -ffp-contract=off keeps every product and sum rounded
separately (the reference's Rust never fuses to FMA, and gcc on aarch64 would
otherwise contract by default); -fopenmp gives the multi-threaded CPU baseline.
No -march=native: the same source must build on x86_64 and aarch64 hosts.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SOURCES = ["drainage.cpp", "interference.cpp", "surrogate.cpp", "shade.cpp", "caustics.cpp", "branched.cpp",
           "foam_dynamics.cpp"]
CXXFLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-Wall"]


def _stale(lib: str, deps: list[str]) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    deps = srcs + [os.path.join(HERE, "oracle.h"), os.path.join(HERE, "..", "include", "sbs_nn.h"),
            os.path.join(HERE, "..", "include", "sbs.h"), __file__]
    if not force and not _stale(LIB, deps):
        return LIB
    cxx = os.environ.get("CXX", "g++")
    objs = []

    def compile_one(src: str) -> str:
        obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
        subprocess.run([cxx, *CXXFLAGS, "-c", src, "-o", obj], check=True)
        return obj

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    subprocess.run([cxx, "-shared", "-fopenmp", "-o", tmp, *objs], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
