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
