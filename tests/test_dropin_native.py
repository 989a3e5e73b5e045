"""The C++ drop-in header: the reference's CPU demo call sequence
(apps/cpu_demo/main.cpp:63-154) compiled unchanged against
include/octree_gb300_kernels.hpp, run on the GPU, must reproduce the
reference's stage hashes for the 1,048,576-point cloud."""
import os
import subprocess

import pytest

from pipeline_gb300 import build as B

pytestmark = pytest.mark.gpu

ROOT = B.ROOT
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def test_dropin_demo_matches_reference_hashes(golden, tmp_path):
    B.build()
    exe = tmp_path / "dropin_demo"
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(CUDA, "include"), os.path.join(ROOT, "tests", "native", "dropin_demo.cpp"),
           "-L", B.OUT_DIR, "-lpipeline_gb300", "-L", os.path.join(CUDA, "lib64"), "-lcudart",
           "-Wl,-rpath," + B.OUT_DIR, "-o", str(exe)]
    subprocess.run(cmd, check=True)
    out = subprocess.run([str(exe), str(golden["cfg1_uniform_1m"]["n"])], check=True,
                         capture_output=True, text=True).stdout
    got = dict(line.split() for line in out.strip().splitlines())
    g = golden["cfg1_uniform_1m"]
    assert int(got["n_unique"]) == g["n_unique"]
    assert int(got["n_oct"]) == g["n_oct"]
    for key, h in g["hashes"].items():
        assert got[key] == h, key
