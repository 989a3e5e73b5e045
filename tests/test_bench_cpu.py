"""bench.py's CPU legs without a GPU: the reference arm (`--impl reference`,
the reference's CPU build on all host threads) prints one well-formed JSON
line, and the GPU arm's CPU baseline reports all cores, one thread and the
per-stage times."""
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["steps"] == 1 and d["value"] > 0
    assert d["unit"] == "Mpoints/s" and d["higher_is_better"] is True
    assert d["config"]["n_points"] == 16_777_216
    assert d["e2e"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1


def test_cpu_baseline_reports_all_cores_one_thread_and_stages():
    sys.path.insert(0, ROOT)
    import bench
    from pipeline_gb300.kernels import k_InitRandomVec4

    pts = np.asarray(k_InitRandomVec4(None, 1 << 16, 0.0, 1024.0, 114514))
    b = bench.cpu_baseline(pts, reps=1)
    assert b["value"] > 0 and b["cores"] >= 1 and b["kind"] == "port"
    assert b["single_thread"]["cores"] == 1 and b["single_thread"]["value"] > 0
    for stages in (b["stages_ms"], b["single_thread"]["stages_ms"]):
        assert list(stages) == bench.CPU_STAGES
        assert all(v >= 0 for v in stages.values())
    assert "65,536-point cloud" in b["sample"]
