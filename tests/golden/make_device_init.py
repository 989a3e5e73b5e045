"""Generate tests/golden/device_init.json from the reference's own device generator.

Runs on a machine with a GB300 and oracle/_ref/init_ref.sm_103a.cubin (built
by oracle/build_ref.sh from the unmodified kernels/cuda/00_init.cu where the
reference sources are; it travels with the repository copy). It loads the
cubin through the CUDA driver API, launches gpu::k_InitRandomVec4 the way the
reference's driver does (apps/gpu_demo/main.cu:168-175: 768 threads a block,
ceil(n / 768) blocks, one element per thread) and records, per case, the
FNV-1a-64 of the n float4 values and the first two points.

Usage: python tests/golden/make_device_init.py [OUT_JSON]
"""
from __future__ import annotations

import ctypes as C
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

CUBIN = os.path.join(ROOT, "oracle", "_ref", "init_ref.sm_103a.cubin")
# gpu::k_InitRandomVec4(glm::vec4*, int, float, float, int), Itanium-mangled.
KERNEL = b"_ZN3gpu16k_InitRandomVec4EPN3glm4vec4Eiffi"
THREADS = 768

# (n, min, range, seed): the driver's cloud (16,777,216 points, seed 114514)
# and the cases of tests/test_consumers_gpu.py.
CASES = [(1 << 24, 0.0, 1024.0, 114514), (1, 0.0, 1024.0, 114514), (767, 0.0, 1024.0, 114514),
         (100_003, 0.0, 1024.0, 114514), (5000, -3.5, 7.25, 1), (4099, 100.0, 0.001, -17),
         (3000, 0.0, 1.0, 0)]


def run_reference(n: int, mn: float, rg: float, seed: int) -> np.ndarray:
    import torch

    torch.cuda.init()
    out = torch.empty((max(n, 1), 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()  # the primary context is current on this thread
    cu = C.CDLL("libcuda.so.1")
    mod, fn = C.c_void_p(), C.c_void_p()
    rc = cu.cuModuleLoad(C.byref(mod), CUBIN.encode())
    assert rc == 0, f"cuModuleLoad: {rc}"
    rc = cu.cuModuleGetFunction(C.byref(fn), mod, KERNEL)
    assert rc == 0, f"cuModuleGetFunction: {rc}"
    a_ptr = C.c_uint64(out.data_ptr())
    a_n, a_min, a_rg, a_seed = C.c_int(n), C.c_float(mn), C.c_float(rg), C.c_int(seed)
    params = (C.c_void_p * 5)(*[C.cast(C.byref(v), C.c_void_p) for v in (a_ptr, a_n, a_min, a_rg, a_seed)])
    grid = (n + THREADS - 1) // THREADS
    rc = cu.cuLaunchKernel(fn, grid, 1, 1, THREADS, 1, 1, 0, None, params, None)
    assert rc == 0, f"cuLaunchKernel: {rc}"
    assert cu.cuCtxSynchronize() == 0
    res = out[:n].cpu().numpy().copy()
    cu.cuModuleUnload(mod)
    return res


def main(argv):
    from oracle import oracle as O

    if not os.path.exists(CUBIN):
        raise SystemExit(f"{CUBIN} is missing: run oracle/build_ref.sh where the reference is")
    dst = argv[0] if argv else os.path.join(HERE, "device_init.json")
    out = {"generator": "tests/golden/make_device_init.py",
           "source": "kernels/cuda/00_init.cu:27-50 run unmodified, launched as apps/gpu_demo/main.cu:168-175",
           "hash": "fnv1a64 over the n float4 values", "cases": []}
    for n, mn, rg, seed in CASES:
        v = run_reference(n, mn, rg, seed)
        out["cases"].append({"n": n, "min": mn, "range": rg, "seed": seed, "hash": O.fnv1a64(v),
                             "first_points": v[:2].tolist()})
        print(out["cases"][-1])
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1:])
