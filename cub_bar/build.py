"""Build recipe for the CUB comparison bar used by bench.py.

CUB's DeviceRadixSort::SortKeys on the same keys as the library's sort (the
library sort the reference benchmarks against,
benchmarks/cuda/bm_02_sort.cuh:117-140), compiled for sm_103a into its own
shared library, cub_bar/_lib/libcub_bar.so. It sits beside the bench, outside
the product package: no product path links or loads it.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cub_sort.cu")
LIB = os.path.join(HERE, "_lib", "libcub_bar.so")


def build(force: bool = False, verbose: bool = False) -> str | None:
    """Returns the library's path, or None when CUB does not build here."""
    from pipeline_gb300.build import ARCH_FLAGS, _stale, nvcc

    if not force and not _stale(LIB, [SRC, os.path.abspath(__file__)]):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [nvcc(), *ARCH_FLAGS, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-cudart",
           "static", SRC, "-o", tmp]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        if verbose:
            sys.stdout.write(r.stdout.decode(errors="replace"))
        return None
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
