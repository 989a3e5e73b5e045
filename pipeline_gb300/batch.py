"""Batched octree build: many clouds of uneven size in one launch sequence.

``BatchOctreeBuilder(sizes)`` plans the batch once (tile descriptors, cloud
offsets, workspace), then ``build(points, mins, ranges)`` builds every cloud;
``capture()``/``replay()`` run the same launches as one CUDA graph.
``shard_clouds`` splits a batch over ranks (independent clouds: no
collective is needed) and ``ShardBuilder`` builds one rank's share of it.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .kernels import OCTNODE_WORDS, oct_nodes_to_numpy


def shard_clouds(sizes, world: int) -> list[list[int]]:
    """Greedy longest-first assignment of clouds to `world` ranks by point
    count (each cloud to the currently lightest rank; ties to the lower rank).
    Deterministic; every cloud appears on exactly one rank."""
    order = sorted(range(len(sizes)), key=lambda c: (-int(sizes[c]), c))
    loads = [0] * world
    out: list[list[int]] = [[] for _ in range(world)]
    for c in order:
        r = min(range(world), key=lambda k: (loads[k], k))
        out[r].append(c)
        loads[r] += int(sizes[c])
    return [sorted(x) for x in out]


def shard_slices(sizes, clouds) -> list[tuple[int, int]]:
    """Row ranges [lo, hi) of the given clouds in the batch's concatenated
    points (clouds stored one after another in index order), in the order
    the clouds are listed."""
    start = np.concatenate([[0], np.cumsum(np.asarray(sizes, np.int64))])
    return [(int(start[c]), int(start[c + 1])) for c in clouds]


def pack_shard(points, mins, ranges, sizes, clouds):
    """The listed clouds' points packed one after another, and their mins and
    ranges. `points` is the whole batch's (N x 4) float32 tensor or a list of
    per-cloud arrays; `mins` and `ranges` hold one value per cloud of the
    batch. Runs on whichever device the inputs are on. Raises ValueError
    when the points do not hold the sizes' rows of 4 values."""
    if isinstance(points, (list, tuple)):
        if len(points) != len(sizes):
            raise ValueError("one array of points per cloud of the batch")
        parts = [torch.as_tensor(points[c]) for c in clouds]
        for c, part in zip(clouds, parts):
            if tuple(part.shape) != (int(sizes[c]), 4):
                raise ValueError(f"cloud {c}: points of shape {tuple(part.shape)}, "
                                 f"expected ({int(sizes[c])}, 4)")
    else:
        points = torch.as_tensor(points)
        total = int(np.sum(np.asarray(sizes, np.int64)))
        if points.dim() != 2 or points.shape[1] != 4 or points.shape[0] < total:
            raise ValueError(f"points of shape {tuple(points.shape)}: expected ({total}, 4)")
        parts = [points[lo:hi] for lo, hi in shard_slices(sizes, clouds)]
    mins = torch.as_tensor(mins, dtype=torch.float32)
    ranges = torch.as_tensor(ranges, dtype=torch.float32)
    idx = torch.as_tensor(list(clouds), dtype=torch.long, device=mins.device)
    pts = torch.cat(parts, 0) if parts else torch.zeros((0, 4), dtype=torch.float32)
    return pts, mins.index_select(0, idx), ranges.index_select(0, idx.to(ranges.device))


class BatchOctreeBuilder:
    """Batched build of clouds of the given sizes. With `model` (a fitted
    LearnedCDF shared by the clouds) stage 2 is the learned bucket sort with
    `n_buckets` buckets per cloud (oct_build_octree_batch_learned)."""

    def __init__(self, sizes, node_caps=None, device="cuda", model=None, n_buckets=None):
        self.lib = _lib.load()
        self.device = torch.device(device)
        self.sizes = np.asarray(sizes, np.int32)
        caps = None if node_caps is None else np.asarray(node_caps, np.int32)
        self.plan = self.lib.oct_batch_plan_create(
            len(self.sizes), self.sizes.ctypes.data, None if caps is None else caps.ctypes.data)
        if not self.plan:
            raise ValueError("oct_batch_plan_create rejected the cloud sizes")
        info = (C.c_int64 * 6)()
        _lib.check(self.lib.oct_batch_plan_info(self.plan, info), "oct_batch_plan_info")
        self.n_clouds, self.n, self.cap, tbytes, wbytes, self.sort_tiles = (int(v) for v in info)
        self.start = np.concatenate([[0], np.cumsum(self.sizes.astype(np.int64))]).astype(np.int64)
        cap_arr = self.sizes if caps is None else caps
        self.node_start = np.concatenate([[0], np.cumsum(cap_arr.astype(np.int64))]).astype(np.int64)
        dev = self.device
        n = max(self.n, 1)
        self.model = model
        self.nb = int(n_buckets or (model.n_buckets if model is not None else 0))
        if model is not None:
            wbytes = self.lib.oct_batch_learned_workspace_bytes(self.plan, self.nb)
            if not wbytes:
                raise ValueError("bad bucket count for the learned batched build")
        self.stats = torch.zeros(12, dtype=torch.int32, device=dev)  # LsortStats
        self.tables = torch.empty(max(tbytes, 256), dtype=torch.uint8, device=dev)
        self.workspace = torch.empty(max(wbytes, 256), dtype=torch.uint8, device=dev)
        self.codes = torch.empty(n, dtype=torch.int32, device=dev)
        self.prefix_n = torch.empty(n, dtype=torch.uint8, device=dev)
        self.has_leaf_left = torch.empty(n, dtype=torch.uint8, device=dev)
        self.has_leaf_right = torch.empty(n, dtype=torch.uint8, device=dev)
        self.left_child = torch.empty(n, dtype=torch.int32, device=dev)
        self.parent = torch.empty(n, dtype=torch.int32, device=dev)
        self.edge_count = torch.empty(n, dtype=torch.int32, device=dev)
        self.prefix_sum = torch.empty(n, dtype=torch.int32, device=dev)
        self.nodes = torch.empty((max(self.cap, 1), OCTNODE_WORDS), dtype=torch.int32, device=dev)
        self.counts = torch.zeros(4 * self.n_clouds, dtype=torch.int32, device=dev)
        self._out = _lib.OctBuildOutputs(
            codes=self.codes.data_ptr(), n_nodes=0, prefix_n=self.prefix_n.data_ptr(),
            has_leaf_left=self.has_leaf_left.data_ptr(), has_leaf_right=self.has_leaf_right.data_ptr(),
            left_child=self.left_child.data_ptr(), parent=self.parent.data_ptr(),
            edge_count=self.edge_count.data_ptr(), prefix_sum=self.prefix_sum.data_ptr(),
            nodes=self.nodes.data_ptr(), nodes_capacity=max(self.cap, 1), d_counts=self.counts.data_ptr())
        s = torch.cuda.current_stream(dev)
        _lib.check(self.lib.oct_batch_upload_tables(self.plan, C.c_void_p(self.tables.data_ptr()),
                                                     C.c_void_p(s.cuda_stream)), "oct_batch_upload_tables")
        self._graph = None

    def __del__(self):
        try:
            if getattr(self, "plan", None):
                self.lib.oct_batch_plan_destroy(self.plan)
                self.plan = None
        except Exception:
            pass

    def build(self, points: torch.Tensor, mins: torch.Tensor, ranges: torch.Tensor,
              stream: torch.cuda.Stream | None = None) -> None:
        if points.numel() < 4 * self.n or not points.is_cuda or points.dtype != torch.float32:
            raise ValueError("points: float32 CUDA tensor of the batch's total size x 4")
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        if self.model is not None:
            rc = self.lib.oct_build_octree_batch_learned(
                self.plan, C.c_void_p(self.tables.data_ptr()), C.c_void_p(points.data_ptr()),
                C.c_void_p(mins.data_ptr()), C.c_void_p(ranges.data_ptr()),
                C.c_void_p(self.model.blob.data_ptr()), self.model.max_segments, self.nb,
                C.byref(self._out), C.c_void_p(self.counts.data_ptr()),
                C.c_void_p(self.stats.data_ptr()), C.c_void_p(self.workspace.data_ptr()),
                self.workspace.numel(), C.c_void_p(s.cuda_stream))
            _lib.check(rc, "oct_build_octree_batch_learned")
            return
        rc = self.lib.oct_build_octree_batch(
            self.plan, C.c_void_p(self.tables.data_ptr()), C.c_void_p(points.data_ptr()),
            C.c_void_p(mins.data_ptr()), C.c_void_p(ranges.data_ptr()), C.byref(self._out),
            C.c_void_p(self.counts.data_ptr()), C.c_void_p(self.workspace.data_ptr()),
            self.workspace.numel(), C.c_void_p(s.cuda_stream))
        _lib.check(rc, "oct_build_octree_batch")

    def same_results(self, other: "BatchOctreeBuilder") -> bool:
        """True when both builders' last builds gave the same counts and, per
        cloud, the same codes [0, U) and OctNodes [0, M) (the rest of each
        cloud's output range is not defined)."""
        if not torch.equal(self.counts, other.counts):
            return False
        counts = self.cloud_counts()
        for c in range(self.n_clouds):
            u, m = int(counts[c][0]), int(counts[c][2])
            cs, ns = int(self.start[c]), int(self.node_start[c])
            if not torch.equal(self.codes[cs:cs + u], other.codes[cs:cs + u]):
                return False
            if not torch.equal(self.nodes[ns:ns + m], other.nodes[ns:ns + m]):
                return False
        return True

    def learned_stats(self) -> dict:
        """Learned stage of the last build: fallback (1 if the LSD passes
        sorted the batch), the largest bucket, buckets per bucket form."""
        v = self.stats.cpu().tolist()
        return {"fallback": int(v[0]), "max_bucket": int(v[3]), "bitmap_buckets": int(v[7]),
                "radix_buckets": int(v[8]), "bitonic_buckets": int(v[9])}

    def capture(self, points, mins, ranges):
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            self.build(points, mins, ranges)
        torch.cuda.current_stream(self.device).wait_stream(s)
        torch.cuda.synchronize(self.device)
        with torch.cuda.graph(g):
            self.build(points, mins, ranges)
        self._graph = g
        return g

    def replay(self):
        self._graph.replay()

    def cloud_counts(self) -> np.ndarray:
        return self.counts.cpu().numpy().reshape(-1, 4)

    def cloud_result(self, c: int, counts: np.ndarray | None = None) -> dict:
        cnt = self.cloud_counts() if counts is None else counts
        u, b, m, st = (int(x) for x in cnt[c])
        cs, ns = int(self.start[c]), int(self.node_start[c])
        out = {"n_unique": u, "n_brt": b, "n_oct": m, "status": st & 0xFFFFFFFF,
               "sorted_unique": self.codes[cs:cs + u].cpu().numpy().view(np.uint32)}
        for name in ("prefix_n", "has_leaf_left", "has_leaf_right", "left_child", "parent",
                     "edge_count", "prefix_sum"):
            out[name] = getattr(self, name)[cs:cs + b].cpu().numpy()
        out["oct_nodes"] = oct_nodes_to_numpy(self.nodes[ns:ns + m]) if m else np.zeros(0)
        return out


class ShardBuilder:
    """One rank's share of a batch split over `world` ranks by shard_clouds:
    the rank builds only its own clouds, as one batched build on its device,
    with no collective on the data path (the clouds are independent). Cloud
    indices (`clouds`, `cloud_result`) are the whole batch's."""

    def __init__(self, sizes, rank: int, world: int, device="cuda", model=None, n_buckets=None):
        if world < 1 or not 0 <= rank < world:
            raise ValueError("rank must lie in [0, world)")
        self.sizes = [int(v) for v in sizes]
        self.rank, self.world = rank, world
        self.clouds = shard_clouds(self.sizes, world)[rank]
        self._local = {c: k for k, c in enumerate(self.clouds)}
        self.n_points = sum(self.sizes[c] for c in self.clouds)
        self.device = torch.device(device)
        self.builder = None
        if self.clouds:
            self.builder = BatchOctreeBuilder([self.sizes[c] for c in self.clouds], device=device,
                                              model=model, n_buckets=n_buckets)
        self._inputs = None

    def select(self, points, mins, ranges):
        """This rank's points, mins and ranges out of the whole batch's,
        packed on the rank's device (a 1 x 4 zero tensor stands in for
        points when the rank's clouds are all empty)."""
        pts, mn, rg = pack_shard(points, mins, ranges, self.sizes, self.clouds)
        if pts.shape[0] == 0:
            pts = torch.zeros((1, 4), dtype=torch.float32)
        dev = self.device
        return (pts.to(dev, torch.float32).contiguous(), mn.to(dev).contiguous(),
                rg.to(dev).contiguous())

    def build(self, points, mins, ranges, stream: torch.cuda.Stream | None = None) -> None:
        """Build this rank's clouds of the batch (whole-batch inputs, see
        `select`). A rank without clouds does nothing."""
        if self.builder is None:
            return
        self._inputs = self.select(points, mins, ranges)  # alive while the build runs
        self.builder.build(*self._inputs, stream=stream)

    def capture(self, points, mins, ranges):
        """Capture this rank's build in a CUDA graph (inputs packed once and
        kept for the replays); None for a rank without clouds."""
        if self.builder is None:
            return None
        self._inputs = self.select(points, mins, ranges)
        return self.builder.capture(*self._inputs)

    def replay(self):
        if self.builder is not None:
            self.builder.replay()

    def cloud_counts(self) -> dict:
        """(U, B, M, status) of each of this rank's clouds, by batch index."""
        if self.builder is None:
            return {}
        cnt = self.builder.cloud_counts()
        return {c: tuple(int(v) for v in cnt[k]) for c, k in self._local.items()}

    def cloud_result(self, c: int) -> dict:
        """Every stage buffer of batch cloud `c`, which must be on this rank."""
        if c not in self._local:
            raise ValueError(f"cloud {c} is not on rank {self.rank}")
        return self.builder.cloud_result(self._local[c])
