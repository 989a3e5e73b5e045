"""Build recipe for the native library libpipeline_gb300.so (in-tree).

Compiles every translation unit under pipeline_gb300/csrc/ with nvcc for
sm_103a only (``-gencode arch=compute_103a,code=sm_103a``), in parallel, and
links them into pipeline_gb300/_lib/libpipeline_gb300.so with the CUDA runtime
linked statically (the library needs only the driver at run time).

Usage: python -m pipeline_gb300.build [--force] [--verbose]
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import time

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(PKG, "_lib")
LIB_NAME = "libpipeline_gb300.so"
LIB_PATH = os.path.join(OUT_DIR, LIB_NAME)

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
    "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr", "-DOCT_BUILT_ARCH=1033", "-I", INCLUDE, "-I", CSRC,
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpipeline_gb300.so")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    srcs = sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    deps = srcs + headers + [os.path.abspath(__file__)]
    if not force and not _stale(LIB_PATH, deps):
        return LIB_PATH
    os.makedirs(os.path.join(OUT_DIR, "obj"), exist_ok=True)
    cc = nvcc()
    t0 = time.time()
    procs = []
    objs = []
    for src in srcs:
        obj = os.path.join(OUT_DIR, "obj", os.path.basename(src) + ".o")
        objs.append(obj)
        cmd = [cc, *ARCH_FLAGS, *NVCC_FLAGS, "-c", src, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
            print(" ".join(cmd), flush=True)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if verbose or p.returncode != 0:
            sys.stdout.write(out.decode(errors="replace"))
        if p.returncode != 0:
            failed.append(src)
    if failed:
        raise RuntimeError("nvcc failed for: " + ", ".join(os.path.basename(f) for f in failed))
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    link = [cc, *ARCH_FLAGS, "-shared", "-cudart", "static", *objs, "-o", tmp]
    subprocess.run(link, check=True)
    os.replace(tmp, LIB_PATH)
    if verbose:
        print(f"built {LIB_PATH} in {time.time() - t0:.1f}s")
    return LIB_PATH


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="--verbose" in sys.argv)
