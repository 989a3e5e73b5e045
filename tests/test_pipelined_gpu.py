"""Pipelined driver (upload / build / download of consecutive frames on three
streams): every frame's OctNodes, read back to the host, equal the oracle's
build of that frame, whatever the order the streams ran in."""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def frames_for(sizes, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i, n in enumerate(sizes):
        pts = rng.random((n, 4), dtype=np.float32) * 1000.0
        if i % 3 == 1:  # clustered frame: many duplicate Morton codes
            pts = np.round(pts / 37.0) * 37.0
        out.append(pts.astype(np.float32))
    return out


@pytest.mark.parametrize("depth", [2, 3])
def test_pipelined_frames_match_oracle(depth):
    from pipeline_gb300.kernels import oct_nodes_to_numpy
    from pipeline_gb300.pipeline import PipelinedBuilder

    sizes = [50_000, 3, 120_000, 1, 80_000, 0, 200_000]
    clouds = frames_for(sizes, seed=depth)
    n_max = max(sizes)
    pb = PipelinedBuilder(n_max, depth=depth)
    frames = [(torch.from_numpy(c).pin_memory(), 0.0, 1000.0) for c in clouds]
    outputs = [torch.zeros((n_max, 15), dtype=torch.int32).pin_memory() for _ in clouds]
    res = pb.run(frames, outputs)
    pb.synchronize()
    assert [r[0] for r in res] == list(range(len(clouds)))
    for (f, u, m, st), c, out in zip(res, clouds, outputs):
        want = O.build_all(c, 0.0, 1000.0, threads=4)
        assert st == 0
        assert u == want["n_unique"] and m == len(want["oct_nodes"])
        got = oct_nodes_to_numpy(out[:m])
        assert got.tobytes() == want["oct_nodes"].tobytes(), f"frame {f}"


def test_pipelined_output_reuse_keeps_last_frames():
    """With fewer output buffers than frames, buffer i holds the last frame
    mapped to it."""
    from pipeline_gb300.kernels import oct_nodes_to_numpy
    from pipeline_gb300.pipeline import PipelinedBuilder

    clouds = frames_for([30_000] * 6, seed=11)
    pb = PipelinedBuilder(30_000, depth=3)
    frames = [(torch.from_numpy(c).pin_memory(), 0.0, 1000.0) for c in clouds]
    outputs = [torch.zeros((30_000, 15), dtype=torch.int32).pin_memory() for _ in range(2)]
    res = pb.run(frames, outputs)
    pb.synchronize()
    for f in (4, 5):
        m = res[f][2]
        want = O.build_all(clouds[f], 0.0, 1000.0, threads=4)["oct_nodes"]
        assert oct_nodes_to_numpy(outputs[f % 2][:m]).tobytes() == want.tobytes()
