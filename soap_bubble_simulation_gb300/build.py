"""Build recipe for libsbs.so, the C-ABI library of CUDA kernels (sm_103a only).

Each translation unit under csrc/ is compiled by nvcc in parallel and linked
into soap_bubble_simulation_gb300/_build/libsbs.so (in-tree, git-ignored).
Flags that matter for parity: -fmad=false stops nvcc from fusing a*b+c on its
own (the kernels spell every fused multiply-add out as fmaf, so the oracle can
repeat them) and -Xcompiler -ffp-contract=off does the same for host code.
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
LIB = os.path.join(OUT_DIR, "libsbs.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-std=c++17",
    "-lineinfo",
    "-fmad=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O3",
    "-Xptxas", "-O3",
    *ARCH,
]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsbs")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps() -> list[str]:
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hdrs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hdrs + [__file__]


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = nvcc_path()
    srcs = sources()
    common = _deps()
    flags = NVCC_FLAGS + list(extra_flags or [])

    def compile_one(src: str) -> str:
        obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
        if force or _stale(obj, [src] + common):
            cmd = [nvcc, *flags, "-I", INCLUDE, "-c", src, "-o", obj]
            if verbose:
                print(" ".join(cmd), flush=True)
            subprocess.run(cmd, check=True)
        return obj

    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(compile_one, srcs))
    if force or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        subprocess.run([nvcc, "-shared", *ARCH, "-o", tmp, *objs], check=True)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
