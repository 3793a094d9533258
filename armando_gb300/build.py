"""In-tree build of the sm_103a library (nvcc, one translation unit)."""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc", "armando.cu")
OUT = os.path.join(HERE, "lib", "libarmando_gb300.so")

NVCC_FLAGS = [
    "-std=c++17", "-O3", "-lineinfo",
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-Xcompiler", "-fPIC", "-shared",
    # host code rounds like the oracle on x86 and on Arm (no fused multiply-add)
    "-Xcompiler", "-ffp-contract=off",
]


def sources():
    csrc = os.path.join(HERE, "csrc")
    return [os.path.join(csrc, f) for f in sorted(os.listdir(csrc))
            if f.endswith((".cu", ".cuh", ".h"))] + [
        os.path.join(os.path.dirname(HERE), "include", "armando.h")]


def up_to_date() -> bool:
    if not os.path.exists(OUT):
        return False
    t = os.path.getmtime(OUT)
    return all(os.path.getmtime(s) <= t for s in sources())


def build_library(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    """Compiles csrc/armando.cu into lib/libarmando_gb300.so (skipped when fresh)."""
    if not force and up_to_date():
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    nvcc = os.environ.get("NVCC", "nvcc")
    cmd = [nvcc, *NVCC_FLAGS, *extra_flags, "-o", OUT, SRC]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    return OUT


if __name__ == "__main__":
    print(build_library(force=True, verbose=True))
