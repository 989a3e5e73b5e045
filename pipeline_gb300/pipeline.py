"""Whole octree build on the device (stages 1-8 in one call).

``OctreeBuilder`` owns the workspace and output buffers for clouds of up to
``n_max`` points and runs ``oct_build_octree``: every size (U, M) stays on
the device, so a build is a fixed launch sequence that can be captured in a
CUDA graph and replayed. This is the reference's apps/cpu_demo/main.cpp:72-154
call sequence with no host round trip between stages.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .kernels import OCTNODE_WORDS, oct_nodes_to_numpy


@dataclass
class BuildCounts:
    n_unique: int
    n_brt: int
    n_oct: int
    status: int


class OctreeBuilder:
    """Device-resident octree build for clouds of up to ``n_max`` points.

    ``nodes_capacity`` bounds the number of OctNodes (default n_max, enough for
    the uniform clouds where M is about 0.48 n); a build that needs more sets
    OCT_STATUS_CAPACITY and reports the needed M in its counts.
    """

    def __init__(self, n_max: int, nodes_capacity: int | None = None, device="cuda"):
        if n_max < 0 or n_max > _lib.OCT_MAX_N:
            raise ValueError("n_max out of range")
        self.lib = _lib.load()
        self.device = torch.device(device)
        self.n_max = int(n_max)
        self.cap = int(nodes_capacity if nodes_capacity is not None else max(n_max, 16))
        n = max(self.n_max, 1)
        dev = self.device
        self.codes = torch.empty(n, dtype=torch.int32, device=dev)
        self.prefix_n = torch.empty(n, dtype=torch.uint8, device=dev)
        self.has_leaf_left = torch.empty(n, dtype=torch.uint8, device=dev)
        self.has_leaf_right = torch.empty(n, dtype=torch.uint8, device=dev)
        self.left_child = torch.empty(n, dtype=torch.int32, device=dev)
        self.parent = torch.empty(n, dtype=torch.int32, device=dev)
        self.edge_count = torch.empty(n, dtype=torch.int32, device=dev)
        self.prefix_sum = torch.empty(n, dtype=torch.int32, device=dev)
        self.nodes = torch.empty((max(self.cap, 1), OCTNODE_WORDS), dtype=torch.int32, device=dev)
        self.d_counts = torch.zeros(4, dtype=torch.int32, device=dev)
        ws_bytes = self.lib.oct_build_workspace_bytes(self.n_max, self.cap)
        self.workspace = torch.empty(max(ws_bytes, 256), dtype=torch.uint8, device=dev)
        self._out = _lib.OctBuildOutputs(
            codes=self.codes.data_ptr(), n_nodes=0, prefix_n=self.prefix_n.data_ptr(),
            has_leaf_left=self.has_leaf_left.data_ptr(), has_leaf_right=self.has_leaf_right.data_ptr(),
            left_child=self.left_child.data_ptr(), parent=self.parent.data_ptr(),
            edge_count=self.edge_count.data_ptr(), prefix_sum=self.prefix_sum.data_ptr(),
            nodes=self.nodes.data_ptr(), nodes_capacity=self.cap, d_counts=self.d_counts.data_ptr())
        self._graph = None
        self._graph_key = None

    @property
    def workspace_bytes(self) -> int:
        return self.workspace.numel()

    def build(self, points: torch.Tensor, min_coord: float, rng: float, n: int | None = None,
              stream: torch.cuda.Stream | None = None) -> None:
        """Launch the whole build on ``stream`` (default: current stream)."""
        if n is None:
            n = points.shape[0]
        if n > self.n_max:
            raise ValueError(f"{n} points exceed the builder's n_max {self.n_max}")
        if not points.is_cuda or points.dtype != torch.float32 or not points.is_contiguous():
            raise TypeError("points must be a contiguous float32 CUDA tensor [n, 4]")
        if points.numel() < 4 * n:
            raise ValueError("points tensor smaller than n x 4")
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        rc = self.lib.oct_build_octree(C.c_void_p(points.data_ptr()), n, min_coord, rng,
                                       C.byref(self._out), C.c_void_p(self.workspace.data_ptr()),
                                       self.workspace.numel(), C.c_void_p(s.cuda_stream))
        _lib.check(rc, "oct_build_octree")
        self._last_n = n

    def sort_form(self) -> int:
        """Form of stages 2-3 in the last build (synchronises): 0 LSD passes,
        1 MSD form, 2 LSD chosen by the device for an uneven cloud."""
        torch.cuda.synchronize(self.device)
        f = C.c_int(-1)
        _lib.check(self.lib.oct_build_sort_form(C.c_void_p(self.workspace.data_ptr()),
                                                getattr(self, "_last_n", self.n_max), self.cap,
                                                C.byref(f)), "oct_build_sort_form")
        return f.value

    def counts(self) -> BuildCounts:
        """Synchronise and read {U, U-1, M, status}."""
        h = self.d_counts.to("cpu")
        u, b, m, st = (int(x) for x in h.tolist())
        return BuildCounts(u, b, m, st & 0xFFFFFFFF)

    def capture(self, points: torch.Tensor, min_coord: float, rng: float, n: int | None = None):
        """Capture one build into a CUDA graph (replay with ``replay()``)."""
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            self.build(points, min_coord, rng, n)  # warm-up outside the graph
        torch.cuda.current_stream(self.device).wait_stream(s)
        torch.cuda.synchronize(self.device)
        with torch.cuda.graph(g):
            self.build(points, min_coord, rng, n)
        self._graph = g
        return g

    def replay(self) -> None:
        if self._graph is None:
            raise RuntimeError("capture() first")
        self._graph.replay()

    def result(self, counts: BuildCounts | None = None) -> dict:
        """Host copies of every stage output (after a build)."""
        c = counts or self.counts()
        u, b, m = c.n_unique, c.n_brt, c.n_oct
        out = {
            "n_unique": u, "n_brt": b, "n_oct": m, "status": c.status,
            "sorted_unique": self.codes[:u].cpu().numpy().view(np.uint32),
            "prefix_n": self.prefix_n[:b].cpu().numpy(),
            "has_leaf_left": self.has_leaf_left[:b].cpu().numpy(),
            "has_leaf_right": self.has_leaf_right[:b].cpu().numpy(),
            "left_child": self.left_child[:b].cpu().numpy(),
            "parent": self.parent[:b].cpu().numpy(),
            "edge_count": self.edge_count[:b].cpu().numpy(),
            "prefix_sum": self.prefix_sum[:b].cpu().numpy(),
        }
        if m <= self.cap:
            out["oct_nodes"] = oct_nodes_to_numpy(self.nodes[:m])
        return out


LSORT_STATS = ("fallback", "failed_buckets", "overflow_keys", "max_bucket", "n", "overflow_frac",
               "skip", "bitmap_buckets", "radix_buckets", "bitonic_buckets")
LSORT_STATS_WORDS = 12


def decode_lsort_stats(t: torch.Tensor) -> dict:
    raw = t.cpu().numpy().view(np.uint32)
    out = {k: int(v) for k, v in zip(LSORT_STATS, raw)}
    out["overflow_frac"] = float(raw[5:6].view(np.float32)[0])
    return out


def lsort_unique(keys: torch.Tensor, model, n_buckets: int | None = None,
                 overflow_threshold: float = 0.05):
    """Sorted unique keys through the learned bucketed sort: (unique, stats)."""
    lib = _lib.load()
    n = keys.numel()
    nb = int(n_buckets or model.n_buckets)
    ws_bytes = lib.oct_lsort_workspace_bytes(n, nb, model.max_segments)
    ws = torch.empty(max(ws_bytes, 256), dtype=torch.uint8, device=keys.device)
    out = torch.empty(max(n, 1), dtype=torch.int32, device=keys.device)
    d_u = torch.zeros(1, dtype=torch.int32, device=keys.device)
    stats = torch.zeros(LSORT_STATS_WORDS, dtype=torch.int32, device=keys.device)
    s = torch.cuda.current_stream(keys.device)
    rc = lib.oct_lsort_unique(C.c_void_p(keys.data_ptr()), n, C.c_void_p(model.blob.data_ptr()),
                              model.max_segments, nb, float(overflow_threshold),
                              C.c_void_p(out.data_ptr()), C.c_void_p(d_u.data_ptr()),
                              C.c_void_p(stats.data_ptr()), C.c_void_p(ws.data_ptr()), ws.numel(),
                              None, C.c_void_p(s.cuda_stream))
    _lib.check(rc, "oct_lsort_unique")
    u = int(d_u.item())
    return out[:u], decode_lsort_stats(stats)


class LearnedOctreeBuilder(OctreeBuilder):
    """Whole build with the learned bucketed sort for stages 2-3."""

    def __init__(self, n_max: int, model, nodes_capacity: int | None = None, device="cuda",
                 n_buckets: int | None = None, overflow_threshold: float = 0.05):
        super().__init__(n_max, nodes_capacity, device)
        self.model = model
        self.nb = int(n_buckets or model.n_buckets)
        self.threshold = float(overflow_threshold)
        ws = self.lib.oct_build_learned_workspace_bytes(self.n_max, self.cap, self.nb,
                                                        model.max_segments)
        self.workspace = torch.empty(max(ws, 256), dtype=torch.uint8, device=self.device)
        self.stats = torch.zeros(LSORT_STATS_WORDS, dtype=torch.int32, device=self.device)

    def build(self, points: torch.Tensor, min_coord: float, rng: float, n: int | None = None,
              stream: torch.cuda.Stream | None = None) -> None:
        if n is None:
            n = points.shape[0]
        if n > self.n_max:
            raise ValueError(f"{n} points exceed the builder's n_max {self.n_max}")
        if not points.is_cuda or points.dtype != torch.float32 or not points.is_contiguous():
            raise TypeError("points must be a contiguous float32 CUDA tensor [n, 4]")
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        rc = self.lib.oct_build_octree_learned(
            C.c_void_p(points.data_ptr()), n, min_coord, rng, C.c_void_p(self.model.blob.data_ptr()),
            self.model.max_segments, self.nb, self.threshold, C.byref(self._out),
            C.c_void_p(self.stats.data_ptr()), C.c_void_p(self.workspace.data_ptr()),
            self.workspace.numel(), C.c_void_p(s.cuda_stream))
        _lib.check(rc, "oct_build_octree_learned")

    def lsort_stats(self) -> dict:
        return decode_lsort_stats(self.stats)


class PipelinedBuilder:
    """Host frames in, host octrees out, with transfers and builds overlapped.

    Three streams (upload, build, download) and ``depth`` buffer slots: the
    upload of frame f+1, the build of frame f and the download of frame f-1's
    OctNodes run at the same time. The host stays one frame ahead: it learns
    a frame's node count from a 16-byte read after its build and then queues
    the download of exactly that many nodes. Frames are (pinned host float32
    [n, 4], min_coord, range); outputs go to pinned host buffers.
    """

    def __init__(self, n_max: int, depth: int = 3, nodes_capacity: int | None = None,
                 device="cuda"):
        self.device = torch.device(device)
        self.depth = int(depth)
        self.slots = []
        for _ in range(self.depth):
            b = OctreeBuilder(n_max, nodes_capacity, self.device)
            self.slots.append({
                "builder": b,
                "points": torch.empty((max(n_max, 1), 4), dtype=torch.float32, device=self.device),
                "counts": torch.zeros(4, dtype=torch.int32).pin_memory(),
                "uploaded": torch.cuda.Event(), "built": torch.cuda.Event(),
                "downloaded": torch.cuda.Event(),
            })
        self.s_up = torch.cuda.Stream(self.device)
        self.s_build = torch.cuda.Stream(self.device)
        self.s_down = torch.cuda.Stream(self.device)
        for sl in self.slots:
            sl["downloaded"].record(self.s_down)

    def _download(self, f, sl, outputs, results):
        sl["built"].synchronize()
        u, b, m, st = (int(v) for v in sl["counts"].tolist())
        out = outputs[f % len(outputs)]
        m_copy = min(m, sl["builder"].cap)  # past capacity: status carries OCT_STATUS_CAPACITY
        if m_copy > out.shape[0]:
            raise ValueError(f"frame {f}: {m_copy} OctNodes exceed the output buffer")
        self.s_down.wait_event(sl["built"])
        with torch.cuda.stream(self.s_down):
            out[:m_copy].copy_(sl["builder"].nodes[:m_copy], non_blocking=True)
        sl["downloaded"].record(self.s_down)
        results.append((f, u, m, st))

    def run(self, frames, outputs) -> list:
        """Build every frame; outputs: pinned host int32 [cap, 15] buffers,
        used round-robin (frame f lands in outputs[f % len(outputs)], so pass
        one buffer per frame to keep them all). Returns [(frame, U, M, status)]
        in frame order; the downloads are complete once ``synchronize()``
        returns."""
        pending = []
        results = []
        for f, (pts_h, mn, rg) in enumerate(frames):
            sl = self.slots[f % self.depth]
            n = pts_h.shape[0]
            self.s_up.wait_event(sl["downloaded"])
            with torch.cuda.stream(self.s_up):
                sl["points"][:n].copy_(pts_h, non_blocking=True)
            sl["uploaded"].record(self.s_up)
            self.s_build.wait_event(sl["uploaded"])
            sl["builder"].build(sl["points"], mn, rg, n, stream=self.s_build)
            with torch.cuda.stream(self.s_build):
                sl["counts"].copy_(sl["builder"].d_counts, non_blocking=True)
            sl["built"].record(self.s_build)
            pending.append((f, sl))
            if len(pending) > 1:
                self._download(*pending.pop(0), outputs, results)
        while pending:
            self._download(*pending.pop(0), outputs, results)
        return results

    def synchronize(self):
        self.s_down.synchronize()
