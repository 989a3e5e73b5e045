"""Autotuner: picks one of the candidate sort shapes by timing, records it,
and builds stay bit-exact under the chosen shape."""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_tune_plain_build_and_stay_exact(tmp_path, golden):
    from pipeline_gb300 import autotune
    from pipeline_gb300.pipeline import OctreeBuilder

    g = golden["cfg1_uniform_1m"]
    pts = torch.from_numpy(O.init_random_vec4(g["n"])).cuda()
    table = str(tmp_path / "tuning.json")
    old = autotune.get_config()
    try:
        def make():
            b = OctreeBuilder(g["n"])
            return lambda: b.build(pts, 0.0, 1024.0)

        res = autotune.tune(make, "plain", g["n"], reps=3, path=table)
        assert tuple(res["config"]) in autotune.CANDIDATES
        assert len(res["all"]) == len(autotune.CANDIDATES)
        assert autotune.get_config() == tuple(res["config"])
        autotune.set_config(old)
        assert autotune.apply_cached("plain", g["n"], path=table) == tuple(res["config"])
        b = OctreeBuilder(g["n"])
        b.build(pts, 0.0, 1024.0)
        r = b.result()
        for key, h in g["hashes"].items():
            if key in r:
                assert O.fnv1a64(r[key]) == h, key
    finally:
        autotune.set_config(old)
