"""Learned CDF model of Morton keys (host side of csrc/learned.cu).

``LearnedCDF`` owns one device buffer holding the model (a 256-byte versioned
header plus its arrays). ``fit`` trains it on the GPU from keys the pipeline
produced; ``buckets`` maps keys to bucket ids with exact integer tables;
``state_dict`` / ``load_state_dict`` persist it (the raw bytes + fit metadata).
"""
from __future__ import annotations

import ctypes as C
import struct

import numpy as np
import torch

from . import _lib

HEADER = struct.Struct("<IIiiiiffi")
MAGIC = 0x4643444C
VERSION = 2
PART_NAMES = ("x", "theta", "adam_m", "adam_v", "y", "grad", "yq", "slope", "lut", "bounds", "blut",
              "total")


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


class LearnedCDF:
    def __init__(self, max_segments: int = 1024, device="cuda"):
        self.lib = _lib.load()
        self.max_segments = int(max_segments)
        offs = (C.c_size_t * len(PART_NAMES))()
        _lib.check(self.lib.oct_lcdf_layout(self.max_segments, offs), "oct_lcdf_layout")
        self.offsets = dict(zip(PART_NAMES, [int(o) for o in offs]))
        self.device = torch.device(device)
        self.blob = torch.zeros(self.offsets["total"], dtype=torch.uint8, device=self.device)
        self.n_buckets = 0

    # ------------------------------------------------------------------ fit --
    def fit(self, sample_keys: torch.Tensor, n_segments: int = 1024, steps: int = 200,
            lr: float = 0.05, n_buckets: int = 4096) -> "LearnedCDF":
        n = sample_keys.numel()
        ws_bytes = self.lib.oct_lcdf_fit_workspace_bytes(n)
        ws = torch.empty(ws_bytes, dtype=torch.uint8, device=self.device)
        rc = self.lib.oct_lcdf_fit(C.c_void_p(sample_keys.data_ptr()), n, int(n_segments), int(steps),
                                   float(lr), int(n_buckets), C.c_void_p(self.blob.data_ptr()),
                                   self.max_segments, C.c_void_p(ws.data_ptr()), ws_bytes, _stream())
        _lib.check(rc, "oct_lcdf_fit")
        self.n_buckets = int(n_buckets)
        return self

    def loss_grad(self, sorted_sample: torch.Tensor):
        """(loss, dL/dtheta) of the current parameters on a sorted sample."""
        k = self.header()["n_knots"]
        grad = torch.zeros(max(k, 1), dtype=torch.float32, device=self.device)
        rc = self.lib.oct_lcdf_loss_grad(C.c_void_p(sorted_sample.data_ptr()), sorted_sample.numel(),
                                         C.c_void_p(self.blob.data_ptr()), self.max_segments,
                                         C.c_void_p(grad.data_ptr()), _stream())
        _lib.check(rc, "oct_lcdf_loss_grad")
        return self.header()["loss"], grad[:k].cpu().numpy()

    def build_tables(self, n_buckets: int):
        rc = self.lib.oct_lcdf_tables(C.c_void_p(self.blob.data_ptr()), self.max_segments,
                                      int(n_buckets), _stream())
        _lib.check(rc, "oct_lcdf_tables")
        self.n_buckets = int(n_buckets)

    def buckets(self, keys: torch.Tensor) -> torch.Tensor:
        out = torch.empty(keys.numel(), dtype=torch.int32, device=self.device)
        rc = self.lib.oct_lcdf_buckets(C.c_void_p(self.blob.data_ptr()), self.max_segments,
                                       C.c_void_p(keys.data_ptr()), keys.numel(),
                                       C.c_void_p(out.data_ptr()), _stream())
        _lib.check(rc, "oct_lcdf_buckets")
        return out

    # ------------------------------------------------------------- access --
    def header(self) -> dict:
        raw = self.blob[:HEADER.size].cpu().numpy().tobytes()
        magic, version, k, kmax, s, steps, loss, z, nb = HEADER.unpack(raw)
        return dict(magic=magic, version=version, n_knots=k, max_knots=kmax, n_sample=s,
                    steps=steps, loss=loss, z=z, n_buckets=nb)

    def part(self, name: str, dtype, count: int) -> np.ndarray:
        off = self.offsets[name]
        nbytes = np.dtype(dtype).itemsize * count
        return self.blob[off:off + nbytes].cpu().numpy().view(dtype).copy()

    def set_theta(self, theta: np.ndarray):
        off = self.offsets["theta"]
        t = torch.from_numpy(np.ascontiguousarray(theta, np.float32).view(np.uint8))
        self.blob[off:off + t.numel()].copy_(t)

    def tables(self) -> dict:
        h = self.header()
        k = h["n_knots"]
        return dict(x=self.part("x", np.uint32, k + 1).astype(np.int64),
                    theta=self.part("theta", np.float32, k),
                    yq=self.part("yq", np.uint32, k + 1).astype(np.int64),
                    slope=self.part("slope", np.uint64, k),
                    n_buckets=h["n_buckets"],
                    bounds=self.part("bounds", np.uint32, max(h["n_buckets"], 0) + 1).astype(np.int64),
                    blut=self.part("blut", np.uint16, (1 << 14) + 1).astype(np.int64))

    # -------------------------------------------------------- persistence --
    def state_dict(self) -> dict:
        return {"format": "pipeline_gb300.LearnedCDF", "version": VERSION,
                "max_segments": self.max_segments, "n_buckets": self.n_buckets,
                "header": self.header(), "blob": self.blob.cpu().numpy().tobytes()}

    @classmethod
    def from_state_dict(cls, sd: dict, device="cuda") -> "LearnedCDF":
        if sd.get("format") != "pipeline_gb300.LearnedCDF" or sd.get("version") != VERSION:
            raise ValueError("not a LearnedCDF state of this version")
        m = cls(sd["max_segments"], device)
        data = torch.frombuffer(bytearray(sd["blob"]), dtype=torch.uint8)
        if data.numel() != m.blob.numel():
            raise ValueError("blob size does not match the layout")
        m.blob.copy_(data)
        m.n_buckets = int(sd["n_buckets"])
        h = m.header()
        if h["magic"] != MAGIC or h["version"] != VERSION:
            raise ValueError("bad model header")
        return m
