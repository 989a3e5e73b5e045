"""Autotuner for the radix-sort shape of the octree builds.

Candidates are the sort configurations the library instantiates: digit width
(10-bit: 3 passes over 30-bit Morton keys; 8-bit: 4 passes), keys per thread
(16 or 24, i.e. tiles of 8192 or 12288 keys with 16 warps) and the tile-offset
scheme (0: decoupled look-back, OneSweep; 1: per-tile histograms + tile scan).
``tune`` times whole builds of the caller's workload under each candidate
with CUDA events, applies the fastest (``oct_set_sort_config``) and records it
in a JSON table keyed by workload kind and size class, so later processes
start from it (``apply_cached``).
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os
import statistics

import torch

from . import _lib

CANDIDATES = [(10, 16, 16, 1), (10, 16, 24, 1), (10, 16, 16, 0), (8, 16, 16, 1), (8, 16, 24, 1),
              (8, 16, 16, 0)]
DEFAULT_TABLE = os.path.join(os.path.expanduser("~"), ".cache", "pipeline_gb300", "sort_tuning.json")


def table_path() -> str:
    return os.environ.get("PIPELINE_GB300_TUNING", DEFAULT_TABLE)


def size_class(n: int) -> str:
    return f"2^{max(0, int(math.log2(max(n, 1))))}"


def get_config() -> tuple:
    out = (C.c_int * 4)()
    _lib.check(_lib.load().oct_get_sort_config(out), "oct_get_sort_config")
    return tuple(int(v) for v in out)


def set_config(cfg) -> None:
    _lib.check(_lib.load().oct_set_sort_config(*[int(v) for v in cfg]), "oct_set_sort_config")


def _load_table(path: str) -> dict:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save_table(path: str, table: dict) -> None:
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + f".tmp{os.getpid()}"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def apply_cached(kind: str, n: int, path: str | None = None) -> tuple | None:
    """Apply a previously tuned configuration for (kind, size class), if any."""
    entry = _load_table(path or table_path()).get(f"{kind}/{size_class(n)}")
    if entry:
        set_config(entry["config"])
        return tuple(entry["config"])
    return None


def tune(make_runner, kind: str, n: int, reps: int = 5, candidates=None, path: str | None = None,
         save: bool = True) -> dict:
    """make_runner() -> zero-argument callable launching one build on the
    current stream; it is rebuilt per candidate because workspace sizes depend
    on the sort shape. Returns {config, ms, all: {config: ms}}."""
    stream = torch.cuda.current_stream()
    results = {}
    old = get_config()
    try:
        for cfg in candidates or CANDIDATES:
            set_config(cfg)
            run = make_runner()
            for _ in range(2):
                run()
            torch.cuda.synchronize()
            ts = []
            for _ in range(reps):
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                run()
                b.record(stream)
                b.synchronize()
                ts.append(a.elapsed_time(b))
            results[tuple(cfg)] = statistics.median(ts)
            del run
    finally:
        set_config(old)
    best = min(results, key=results.get)
    set_config(best)
    out = {"config": list(best), "ms": results[best],
           "all": {",".join(map(str, k)): v for k, v in results.items()}}
    if save:
        p = path or table_path()
        table = _load_table(p)
        table[f"{kind}/{size_class(n)}"] = out
        _save_table(p, table)
    return out
