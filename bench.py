"""Octree-build benchmark (one JSON line on rank 0).

Workload (default): the 16,777,216-point uniform cloud in [0,1024)^3 of seed
114514 (the reference's k_InitRandomVec4 stream), all eight stages: Morton
encode, radix sort, unique, Karras radix tree, edge count, prefix sum, octree
nodes and leaf links. One step = one whole build of that cloud.

  value  Mpoints/s with the points already resident in HBM, timed with CUDA
         events around each step (L2 flushed between steps; the 256 MiB input
         is also larger than L2);
  e2e    the same metric through the public API (PipelinedBuilder over the
         C ABI), each step copying its points host->device from pinned
         memory and its octree (M OctNodes + counts) back; consecutive steps'
         uploads, builds and downloads overlap on three streams
         (serial_value: the same with no overlap);
  roofline  the dominant kernel's algorithmic bytes per launch over its
         average duration (CUDA events recorded by oct_build_octree_timed on
         the launching stream), against MEASURED_PEAKS.json's HBM copy rate;
  cpu_baseline  the CPU port of the reference pipeline (oracle/oracle.c,
         OpenMP on all host cores) timed on the same cloud.

--impl reference times that CPU implementation alone (the reference's own
sources cannot be built on the GPU host; the restatement is pinned to them
byte for byte by tests/test_oracle_golden.py).

Multi-GPU: one process per GPU (torchrun). A single cloud does not shard, so
N ranks build N independent replicas (weak scaling); value = all points built
by all ranks / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mpoints/s octree build, learned+batched vs plain GPU (bit-exact); % HBM peak"
UNIT = "Mpoints/s"
N_POINTS = 1 << 24
SEED = 114514
MIN_COORD, RANGE = 0.0, 1024.0
WORKLOAD = ("uniform_16m: 16,777,216 float32 points uniform in [0,1024)^3, seed 114514 "
            "(k_InitRandomVec4 stream), 30-bit Morton, all stages Morton..leaf links")

# Algorithmic bytes per kernel launch of the build (per point / node / slot),
# as fixed by the octree-build analysis: stage 1 reads 16 B and writes 4 B per
# point (its digit histograms are fused, so the sort reads no extra 4 B/key);
# each 10-bit sort pass reads and writes 4 B per key; unique reads 4 B per key
# and writes 4 B per unique key (in the MSD form of large even clouds: pass 0
# scatters on the top digit, 8 B per key, the bucket bitmaps reading 4 B per key and
# writing 4 B per unique key, and the pack reading 4 B and writing 5 B per
# unique key: code and delta); the radix tree with its edge counts reads 4 B
# per code and writes 15 B per node (11 B of tree + 4 B of edge count); the
# prefix sum reads 4 B and writes 4 B per node; octree: 40 B per radix node read, 60 B per OctNode written, 4 B per
# leaf link (split over the emit and finalize launches).
def algorithmic_bytes(n, u, b, m, msd=False):
    leaves = b + 1
    if msd:  # MSD form: pass 0's launches scatter on the top digit, bucket bitmaps, pack
        sort = {"sort pass 0": 8 * n, "msd buckets": 4 * n + 4 * u, "unique": 9 * u}
    else:
        sort = {"sort pass 0": 8 * n, "sort pass 1": 8 * n, "sort pass 2": 8 * n,
                "unique": 4 * n + 4 * u}
    return {
        "morton+histogram": 20 * n,
        **sort,
        "radix tree+edge count": 4 * u + 15 * b,
        "prefix sum": 8 * b,
        "octree emit": 40 * b + 4 * leaves,
        "octree finalize": 60 * m,
    }


def cloud_bytes(counts) -> int:
    """Algorithmic bytes of building clouds whose counts are (n, U, U-1, M)
    rows: the LSD-form accounting of algorithmic_bytes, summed over clouds
    (every form of stages 2-3 produces the same outputs)."""
    return int(sum(sum(algorithmic_bytes(int(n), int(u), int(b), int(m)).values())
                   for n, u, b, m in counts))


def hbm_frac(nbytes: int, ms: float | None):
    """nbytes moved in ms, as a fraction of the measured HBM copy peak."""
    if not ms:
        return None
    return round(nbytes / (ms * 1e-3) / (peaks()[0] * 1e9), 4)


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self._t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self._t:
            self._t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_points(n):
    from pipeline_gb300.kernels import k_InitRandomVec4

    return k_InitRandomVec4(None, n, MIN_COORD, RANGE, SEED)


# ----------------------------------------------------------------- CPU side --
def cpu_build_time(pts, threads, reps):
    """Seconds per whole CPU build (stages 1-8, OpenMP as the reference)."""
    from oracle import oracle as O

    times, r = [], None
    for _ in range(reps):
        r = O.build_all(pts, MIN_COORD, RANGE, threads=threads, parallel_octree=threads > 1,
                        keep_morton=False)
        times.append(float(np.sum(r["stage_ms"])) / 1e3)
    return times, r


def cpu_baseline(pts, reps=2):
    from oracle import oracle as O

    threads = O.lib().orc_max_threads()
    times, r = cpu_build_time(pts, threads, reps)
    t = statistics.median(times)
    # the same CPU path on one thread (the reference run with OMP_NUM_THREADS=1)
    (t1,), r1 = cpu_build_time(pts, 1, 1)
    return {"value": len(pts) / t / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{reps} whole builds of the {len(pts):,}-point cloud, median "
                      f"{t * 1e3:.0f} ms each (stages 1-8; octree stage multi-threaded as in the "
                      f"reference)",
            "stages_ms": cpu_stage_ms(r),
            "single_thread": {"value": len(pts) / t1 / 1e6, "unit": UNIT, "cores": 1,
                              "sample": f"1 whole build of the same cloud on one thread, "
                                        f"{t1 * 1e3:.0f} ms",
                              "stages_ms": cpu_stage_ms(r1)}}


CPU_STAGES = ["morton", "sort", "unique", "radix tree", "edge count", "prefix sum",
              "make octnodes", "link leaf nodes"]


def cpu_stage_ms(r):
    """Per-stage wall times (ms) of one CPU build (the reference's eight stage
    calls, kernels/01_morton.cpp ... 07_octree.cpp)."""
    return {k: round(float(v), 2) for k, v in zip(CPU_STAGES, r["stage_ms"])}


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    from oracle import oracle as O

    pts = make_points(N_POINTS)
    threads = O.lib().orc_max_threads()
    cpu_build_time(pts, threads, max(args.warmup, 0))
    times, _ = cpu_build_time(pts, threads, args.steps)
    total = float(sum(times))
    value = N_POINTS * args.steps / total / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic", "config": {"workload": WORKLOAD, "n_points": N_POINTS},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} whole builds of the workload (after "
                                   f"{args.warmup} warm-up builds) on {threads} host threads; "
                                   "the reference's sources do not build on the GPU host, the "
                                   "timed code is their byte-identical C restatement"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------- GPU side --
def run_ours(args, rank, world, local_rank):
    import torch
    import torch.distributed as dist

    from pipeline_gb300 import _lib
    from pipeline_gb300.pipeline import OctreeBuilder

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    lib = _lib.load()
    pts_h = make_points(N_POINTS)
    pts = torch.from_numpy(pts_h).to(dev)
    builder = OctreeBuilder(N_POINTS, device=dev)
    stream = torch.cuda.current_stream(dev)

    # L2 flush buffer (larger than the 129 MB L2).
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize(dev)

    # warm-up (also records the sizes)
    for _ in range(max(args.warmup, 3)):
        builder.build(pts, MIN_COORD, RANGE)
    counts = builder.counts()
    if counts.status != 0:
        raise RuntimeError(f"device status {counts.status}")
    n, u, b, m = N_POINTS, counts.n_unique, counts.n_brt, counts.n_oct

    # ---- device-resident timing (value) ----
    # A step is one build captured once in a CUDA graph (OctreeBuilder.capture)
    # and replayed: the same launches without the gaps between them. The same
    # build launched kernel by kernel on the stream is timed too (stream_ms).
    builder.capture(pts, MIN_COORD, RANGE)
    for _ in range(2):
        builder.replay()

    def timed_steps(step):
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        for k in range(args.steps):
            flush.fill_(k & 0xFF)
            starts[k].record(stream)
            step()
            ends[k].record(stream)
        barrier()
        return [s.elapsed_time(e) for s, e in zip(starts, ends)]

    barrier()
    stream_step_ms = timed_steps(lambda: builder.build(pts, MIN_COORD, RANGE))
    stream_ms = sum(stream_step_ms) / len(stream_step_ms)
    sampler = ClockSampler(local_rank)
    barrier()
    sampler.start()
    time.sleep(0.25)
    t_wall = time.perf_counter()
    step_ms = timed_steps(builder.replay)
    t_wall = time.perf_counter() - t_wall
    clocks = sampler.stop()
    if builder.counts().status != 0:
        raise RuntimeError("device status after the timed replays")
    ms = sum(step_ms) / len(step_ms)
    if world > 1:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = n * world / (ms / 1e3) / 1e6

    # ---- per-kernel times (timed build, events on the launching stream) ----
    nsteps = lib.oct_build_step_count()
    names = [lib.oct_build_step_name(i).decode() for i in range(nsteps)]
    reps = max(3, min(args.steps, 10))
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(nsteps)] for _ in range(reps)]
    for row in evs:  # torch creates the CUDA event on its first record
        for e in row:
            e.record(stream)
    torch.cuda.synchronize(dev)
    for r in range(reps):
        flush.fill_(r & 0xFF)
        handles = (C.c_void_p * nsteps)(*[e.cuda_event for e in evs[r]])
        rc = lib.oct_build_octree_timed(C.c_void_p(pts.data_ptr()), n, MIN_COORD, RANGE,
                                        C.byref(builder._out), C.c_void_p(builder.workspace.data_ptr()),
                                        builder.workspace.numel(), handles, nsteps,
                                        C.c_void_p(stream.cuda_stream))
        _lib.check(rc, "oct_build_octree_timed")
    torch.cuda.synchronize(dev)
    per_kernel = {}
    for i in range(1, nsteps):
        per_kernel[names[i]] = statistics.median(evs[r][i - 1].elapsed_time(evs[r][i]) for r in range(reps))
    # the MSD form ran when its bucket stage did work (its kernels otherwise
    # return at once)
    msd_form = per_kernel.get("msd buckets", 0.0) > 0.005
    alg = algorithmic_bytes(n, u, b, m, msd_form)
    hbm_peak, peak_kind = peaks()
    stages = {}
    for name, t in per_kernel.items():
        entry = {"ms": round(t, 4)}
        if name in alg and t > 0:
            gbs = alg[name] / (t / 1e3) / 1e9
            entry.update(gbs=round(gbs, 1), frac=round(gbs / hbm_peak, 3))
        stages[name] = entry
    dom = max((k for k in per_kernel if k in alg), key=lambda k: per_kernel[k])
    dom_gbs = alg[dom] / (per_kernel[dom] / 1e3) / 1e9
    traffic = read_traffic(dom, n)
    total_alg = sum(alg.values())
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(dom_gbs, 1), "peak": hbm_peak,
                "unit": "GB/s", "frac": round(dom_gbs / hbm_peak, 4), "traffic": traffic,
                "peak_source": f"{peak_kind} hbm_gbs (MEASURED_PEAKS.json)" if peak_kind == "measured"
                else "fallback 6800 GB/s",
                "end_to_end_frac": round(total_alg / (ms / 1e3) / 1e9 / hbm_peak, 4),
                "algorithmic_bytes_per_step": int(total_alg)}

    # ---- end to end through the C ABI with host buffers (e2e) ----
    pinned = torch.from_numpy(pts_h).pin_memory()
    nodes_h = torch.empty((m, 15), dtype=torch.int32).pin_memory()
    counts_h = torch.empty(4, dtype=torch.int32).pin_memory()
    e2e_steps = max(3, min(args.steps, 10))
    es = [torch.cuda.Event(enable_timing=True) for _ in range(e2e_steps)]
    ee = [torch.cuda.Event(enable_timing=True) for _ in range(e2e_steps)]
    barrier()
    for k in range(e2e_steps):
        flush.fill_(k & 0xFF)
        es[k].record(stream)
        pts.copy_(pinned, non_blocking=True)
        builder.build(pts, MIN_COORD, RANGE)
        counts_h.copy_(builder.d_counts, non_blocking=True)
        nodes_h.copy_(builder.nodes[:m], non_blocking=True)
        ee[k].record(stream)
    barrier()
    e2e_ms = statistics.mean(s.elapsed_time(e) for s, e in zip(es, ee))
    if world > 1:
        t = torch.tensor([e2e_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
    assert int(counts_h[2]) == m
    serial_mpts = n * world / (e2e_ms / 1e3) / 1e6

    # Pipelined through the same public API: three streams, three slots; every
    # step still uploads its points and downloads its OctNodes + counts.
    from pipeline_gb300.pipeline import PipelinedBuilder

    del builder
    torch.cuda.empty_cache()
    pb = PipelinedBuilder(n, depth=3, device=dev)
    outs = [torch.empty((m, 15), dtype=torch.int32).pin_memory() for _ in range(3)]
    frames = [(pinned, MIN_COORD, RANGE)] * e2e_steps
    pb.run(frames[:3], outs)
    pb.synchronize()
    barrier()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(pb.s_up)
    res = pb.run(frames, outs)
    t_end.record(pb.s_down)
    t_end.synchronize()
    pipe_ms = t_start.elapsed_time(t_end) / e2e_steps
    if world > 1:
        t = torch.tensor([pipe_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        pipe_ms = float(t.item())
    assert all(r[2] == m and r[3] == 0 for r in res)
    del pb
    link = host_link_bound(dev, pinned, outs[0], n * 16, m * 60)
    e2e = {"value": n * world / (pipe_ms / 1e3) / 1e6, "unit": UNIT, "h2d_bytes_per_step": n * 16,
           "d2h_bytes_per_step": m * 60 + 16, "ms_per_step": round(pipe_ms, 4),
           "mode": "pipelined: upload, build and download of consecutive steps overlap "
                   "(3 streams, 3 slots)",
           "serial_value": round(serial_mpts, 2), "serial_ms_per_step": round(e2e_ms, 4),
           "link": dict(link, frac=round(link["both_ms"] / pipe_ms, 3))}
    del outs

    workloads = {}
    if not args.no_extra:
        torch.cuda.empty_cache()
        workloads["clustered_16m"] = clustered_workload(dev, flush, max(5, min(args.steps, 20)))
        torch.cuda.empty_cache()
        workloads["batched_512"] = batched_workload(dev, flush, max(5, min(args.steps, 20)))
        torch.cuda.empty_cache()
        workloads["sort_vs_cub"] = sort_bar_workload(dev, flush, max(5, min(args.steps, 20)), pts)
        torch.cuda.empty_cache()
        workloads["frames_224"] = frames_workload(dev, flush, max(5, min(args.steps, 20)))
    if rank != 0:
        return 0
    base = None
    if world == 1 and not args.no_cpu_baseline:
        base = cpu_baseline(pts_h)
    launches_per_step = build_launches(n)
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "n_points": n, "n_unique": u, "n_oct_nodes": m,
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "flushed between steps (256 MiB write); input 256 MiB > L2",
                   "step": "one build captured in a CUDA graph, replayed per step",
                   "stream_launched_ms_per_step": round(stream_ms, 4),
                   "wall_s_timed_region": round(t_wall, 3)},
        "roofline": roofline, "stages": stages, "e2e": e2e,
        "gpu_launches": launches_per_step * args.steps, "clocks": clocks,
        "cpu_baseline": base, "workloads": workloads,
    }
    print(json.dumps(line), flush=True)
    return 0


def host_link_bound(dev, pinned_in, pinned_out, in_bytes: int, out_bytes: int) -> dict:
    """The host link alone, on one step's bytes: the points upload, the
    OctNode download, and both at once on two streams (the pipelined
    end-to-end step's floor). Best of 5 after 2 warm-up copies."""
    import torch

    src = pinned_in.view(-1).view(torch.uint8)[:in_bytes]
    dst_h = pinned_out.view(-1).view(torch.uint8)[:out_bytes]
    d_in = torch.empty(in_bytes, dtype=torch.uint8, device=dev)
    d_out = torch.zeros(out_bytes, dtype=torch.uint8, device=dev)
    s_a, s_b = torch.cuda.Stream(dev), torch.cuda.Stream(dev)

    def timed(fn):
        best = float("inf")
        for r in range(7):
            torch.cuda.synchronize(dev)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            e1.synchronize()
            if r >= 2:
                best = min(best, e0.elapsed_time(e1))
        return best

    def both():
        cur = torch.cuda.current_stream(dev)
        s_a.wait_stream(cur)
        s_b.wait_stream(cur)
        with torch.cuda.stream(s_a):
            d_in.copy_(src, non_blocking=True)
        with torch.cuda.stream(s_b):
            dst_h.copy_(d_out, non_blocking=True)
        cur.wait_stream(s_a)
        cur.wait_stream(s_b)

    h2d = timed(lambda: d_in.copy_(src, non_blocking=True))
    d2h = timed(lambda: dst_h.copy_(d_out, non_blocking=True))
    both_ms = timed(both)
    del d_in, d_out
    return {"h2d_ms": round(h2d, 4), "h2d_gbs": round(in_bytes / h2d / 1e6, 1),
            "d2h_ms": round(d2h, 4), "d2h_gbs": round(out_bytes / d2h / 1e6, 1),
            "both_ms": round(both_ms, 4), "both_gbs": round((in_bytes + out_bytes) / both_ms / 1e6, 1)}


def build_launches(n: int = 0) -> int:
    """Kernel launches of one plain build under the active sort shape:
    Morton, digit-base scan, per pass (tile histogram + tile scan +) pass,
    unique (run-head count, their scan, compaction with the deltas), tree
    nodes, tile-sum scan + prefix sum (which clears the octree tags), octree
    emit/finalize, counts."""
    from pipeline_gb300 import autotune

    rb, _, _, scan = autotune.get_config()
    passes = (30 + rb - 1) // rb
    lsd = 2 + passes * (3 if scan == 1 else 1) + 3 + 1 + 2 + 2 + 1
    # MSD form (launched beside the LSD passes for clouds of 2^22+ points; pass
    # 0's launches double as its top-digit scatter): form gate, bucket
    # bitmaps, pack scan + pack
    msd = 4 if (n >= (1 << 22) and rb == 10 and passes == 3 and scan == 1) else 0
    return lsd + msd


def profile_only(args):
    """--warmup builds then exactly one more build of the workload: a short,
    fixed launch sequence for ncu (build_launches() kernel launches per build)."""
    import torch

    from pipeline_gb300.pipeline import OctreeBuilder

    n = int(args.points)
    if args.profile_only == "batched":
        # the 512-cloud batch of the batched_512 workload (--points unused)
        from pipeline_gb300 import datasets
        from pipeline_gb300.batch import BatchOctreeBuilder

        clouds = datasets.batched(512, seed=11)
        sizes = [len(c) for c in clouds]
        pts = torch.from_numpy(np.concatenate(clouds, 0)).cuda()
        mins = torch.zeros(len(clouds), dtype=torch.float32, device="cuda")
        ranges = torch.full((len(clouds),), RANGE, dtype=torch.float32, device="cuda")
        bb = BatchOctreeBuilder(sizes)
        for _ in range(max(args.warmup, 0) + 1):
            bb.build(pts, mins, ranges)
        torch.cuda.synchronize()
        print(f"profile build (batched): {len(sizes)} clouds, {sum(sizes)} points")
        return 0
    if args.profile_only == "learned":
        # clustered cloud of n points, model fit on 2^18 of its Morton codes
        from pipeline_gb300 import datasets
        from pipeline_gb300.kernels import k_ComputeMortonCode
        from pipeline_gb300.learned import LearnedCDF
        from pipeline_gb300.pipeline import LearnedOctreeBuilder

        pts = torch.from_numpy(datasets.clustered(n, seed=7)).cuda()
        s_n = min(n, 1 << 18)
        idx = torch.from_numpy(np.random.default_rng(1).integers(0, n, s_n)).cuda()
        sk = torch.empty(s_n, dtype=torch.int32, device="cuda")
        k_ComputeMortonCode(pts.index_select(0, idx).contiguous(), sk, s_n, MIN_COORD, RANGE)
        model = LearnedCDF(max_segments=4096).fit(sk, n_segments=4096, steps=0, n_buckets=4096)
        b = LearnedOctreeBuilder(n, model)
    elif args.profile_only == "clustered":
        # plain build of the clustered cloud of n points (uneven top digits:
        # stages 2-3 take the LSD form)
        from pipeline_gb300 import datasets

        pts = torch.from_numpy(datasets.clustered(n, seed=7)).cuda()
        b = OctreeBuilder(n)
    else:
        pts = torch.from_numpy(make_points(n)).cuda()
        b = OctreeBuilder(n)
    for _ in range(max(args.warmup, 0) + 1):
        b.build(pts, MIN_COORD, RANGE)
    torch.cuda.synchronize()
    c = b.counts()
    print(f"profile build ({args.profile_only}): U={c.n_unique} M={c.n_oct} status={c.status}")
    return 0 if c.status == 0 else 1


def _time_events(fn, reps, stream, flush):
    import torch

    ts = []
    for r in range(reps):
        flush.fill_(r & 0xFF)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        b.synchronize()
        ts.append(a.elapsed_time(b))
    return statistics.median(ts)


def _graph_of(fn, dev):
    """fn's launches captured once in a CUDA graph (after one eager run);
    returns the graph's replay, or None when the launches cannot be captured."""
    import torch

    try:
        s = torch.cuda.Stream(dev)
        s.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(s):
            fn()
        torch.cuda.current_stream(dev).wait_stream(s)
        torch.cuda.synchronize(dev)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            fn()
        torch.cuda.synchronize(dev)
        return g.replay
    except Exception:  # pragma: no cover - reported as null
        torch.cuda.synchronize(dev)
        return None


def clustered_workload(dev, flush, reps):
    """16,777,216-point clustered cloud: learned bucketed sort vs plain."""
    import torch

    from pipeline_gb300 import datasets
    from pipeline_gb300.kernels import k_ComputeMortonCode
    from pipeline_gb300.learned import LearnedCDF
    from pipeline_gb300.pipeline import LearnedOctreeBuilder, OctreeBuilder

    n = N_POINTS
    pts_h = datasets.clustered(n, seed=7)
    pts = torch.from_numpy(pts_h).to(dev)
    stream = torch.cuda.current_stream(dev)
    # the model is fit on Morton codes the pipeline produced for a sample of points
    idx = torch.from_numpy(np.random.default_rng(1).integers(0, n, 1 << 18)).to(dev)
    sample_pts = pts.index_select(0, idx).contiguous()
    sample_keys = torch.empty(1 << 18, dtype=torch.int32, device=dev)
    k_ComputeMortonCode(sample_pts, sample_keys, 1 << 18, MIN_COORD, RANGE)
    model = LearnedCDF(max_segments=4096)
    t0 = time.perf_counter()
    model.fit(sample_keys, n_segments=4096, steps=100, lr=0.05, n_buckets=4096)
    torch.cuda.synchronize(dev)
    fit_ms = (time.perf_counter() - t0) * 1e3
    plain = OctreeBuilder(n, device=dev)
    learned = LearnedOctreeBuilder(n, model, device=dev)
    for _ in range(3):
        plain.build(pts, MIN_COORD, RANGE)
        learned.build(pts, MIN_COORD, RANGE)
    torch.cuda.synchronize(dev)
    pc, lc = plain.counts(), learned.counts()
    exact = (pc.n_unique, pc.n_oct) == (lc.n_unique, lc.n_oct) and torch.equal(
        plain.nodes[: pc.n_oct], learned.nodes[: lc.n_oct]) and torch.equal(
        plain.codes[: pc.n_unique], learned.codes[: lc.n_unique])
    t_plain = _time_events(lambda: plain.build(pts, MIN_COORD, RANGE), reps, stream, flush)
    t_learned = _time_events(lambda: learned.build(pts, MIN_COORD, RANGE), reps, stream, flush)
    # the same builds replayed from CUDA graphs (as the headline step is)
    plain_g = _graph_of(lambda: plain.build(pts, MIN_COORD, RANGE), dev)
    learned_g = _graph_of(lambda: learned.build(pts, MIN_COORD, RANGE), dev)
    t_plain_g = _time_events(plain_g, reps, stream, flush) if plain_g else None
    t_learned_g = _time_events(learned_g, reps, stream, flush) if learned_g else None
    st = learned.lsort_stats()
    h = model.header()
    alg = cloud_bytes([(n, pc.n_unique, pc.n_brt, pc.n_oct)])
    return {"workload": "clustered_16m: 64 anisotropic Gaussians (sigma 0.5-20% of the box) + 5% "
                        "uniform noise, 16,777,216 points, seed 7",
            "n_unique": pc.n_unique, "plain_mpts": round(n / t_plain / 1e3, 1),
            "learned_mpts": round(n / t_learned / 1e3, 1),
            "speedup": round(t_plain / t_learned, 3),
            "plain_graph_mpts": round(n / t_plain_g / 1e3, 1) if t_plain_g else None,
            "learned_graph_mpts": round(n / t_learned_g / 1e3, 1) if t_learned_g else None,
            "speedup_graph": round(t_plain_g / t_learned_g, 3) if t_plain_g and t_learned_g else None,
            "hbm_frac_lsd_bytes": {"plain": hbm_frac(alg, t_plain), "learned": hbm_frac(alg, t_learned),
                                   "plain_graph": hbm_frac(alg, t_plain_g),
                                   "learned_graph": hbm_frac(alg, t_learned_g)},
            "bit_exact": bool(exact),
            "overflow_frac": round(st["overflow_frac"], 5), "fallback": st["fallback"],
            "max_bucket": st["max_bucket"], "fit_loss": h["loss"], "fit_ms": round(fit_ms, 2),
            "fit": "4096 segments, 262,144 sampled Morton codes, 100 Adam steps"}


def batched_workload(dev, flush, reps):
    """512 clouds (log-uniform 1K-1M points): one batched sequence vs a
    per-cloud plain loop."""
    import torch

    from pipeline_gb300 import autotune, datasets
    from pipeline_gb300.batch import BatchOctreeBuilder
    from pipeline_gb300.pipeline import OctreeBuilder

    clouds = datasets.batched(512, seed=11)
    sizes = [len(c) for c in clouds]
    total = int(sum(sizes))
    stream = torch.cuda.current_stream(dev)
    pts = torch.from_numpy(np.concatenate(clouds, 0)).to(dev)
    mins = torch.zeros(len(clouds), dtype=torch.float32, device=dev)
    ranges = torch.full((len(clouds),), RANGE, dtype=torch.float32, device=dev)
    # sort shape for this batch chosen by the autotuner (batched plans use the
    # tile-scan offsets, so only those candidates apply)
    old_cfg = autotune.get_config()

    def make_runner():
        bb = BatchOctreeBuilder(sizes, device=dev)
        return lambda: bb.build(pts, mins, ranges)

    tuned = autotune.tune(make_runner, "batched", total, reps=3,
                          candidates=[c for c in autotune.CANDIDATES if c[3] == 1], save=False)
    b = BatchOctreeBuilder(sizes, device=dev)
    b.capture(pts, mins, ranges)
    offs = np.concatenate([[0], np.cumsum(sizes)])
    single = OctreeBuilder(max(sizes), device=dev)
    views = [pts[offs[c]:offs[c + 1]] for c in range(len(clouds))]

    def loop():
        for v in views:
            single.build(v, MIN_COORD, RANGE)

    loop()
    b.replay()
    torch.cuda.synchronize(dev)
    # bit-exactness spot check against the per-cloud build
    counts = b.cloud_counts()
    exact = True
    for c in range(0, 512, 51):
        single.build(views[c], MIN_COORD, RANGE)
        r = single.result()
        g = b.cloud_result(c, counts)
        exact &= r["oct_nodes"].tobytes() == g["oct_nodes"].tobytes()
    t_batch = _time_events(b.replay, reps, stream, flush)
    alg = cloud_bytes([(sz, u, bb, m) for sz, (u, bb, m, _) in zip(sizes, counts)])
    # the same build with its octree-stage kernels fed by a work queue of
    # persistent CTAs instead of one CTA per tile
    from pipeline_gb300 import _lib

    _lib.load().oct_set_batch_work_queue(1)
    b_queue = BatchOctreeBuilder(sizes, device=dev)
    b_queue.capture(pts, mins, ranges)
    _lib.load().oct_set_batch_work_queue(0)
    t_queue = _time_events(b_queue.replay, reps, stream, flush)
    del b_queue
    t_loop = _time_events(loop, max(2, reps // 4), stream, flush)
    e2e = batches_e2e({"batched": b}, {"per_cloud_plain": single}, pts, np.concatenate(clouds, 0),
                      sizes, [MIN_COORD] * len(sizes), [RANGE] * len(sizes), stream, flush,
                      max(2, reps // 4))
    loop_graph = _graph_of(loop, dev)
    t_loop_graph = _time_events(loop_graph, max(2, reps // 4), stream, flush) if loop_graph else None
    autotune.set_config(old_cfg)
    return {"workload": "batched_512: 512 clouds, sizes log-uniform in [1K, 1M] (seed 11), even "
                        "uniform, odd 8-Gaussian mixtures; one CUDA-graph-captured batched build",
            "total_points": total, "batched_mpts": round(total / t_batch / 1e3, 1),
            "batched_hbm_frac_lsd_bytes": hbm_frac(alg, t_batch),
            "batched_work_queue_mpts": round(total / t_queue / 1e3, 1),
            "per_cloud_loop_mpts": round(total / t_loop / 1e3, 1),
            "speedup": round(t_loop / t_batch, 3),
            "per_cloud_loop_graph_mpts": round(total / t_loop_graph / 1e3, 1) if t_loop_graph else None,
            "speedup_vs_graph_loop": round(t_loop_graph / t_batch, 3) if t_loop_graph else None,
            "bit_exact_spot_check": bool(exact),
            "e2e": e2e,
            "autotuned_sort_shape": {"radix_bits": tuned["config"][0], "warps": tuned["config"][1],
                                     "items": tuned["config"][2], "candidates_ms": tuned["all"]}}


def frames_workload(dev, flush, reps):
    """Scan-like frames (64 beams x 1,920 azimuth steps, ground plane + 40
    boxes, 2 cm range noise; per-frame min/range): frames 32-255 built in one
    batched launch sequence vs a per-frame loop, and per frame with a learned
    CDF fit only on frames 0-31's Morton codes (model transfer across frames)
    vs the plain per-frame build."""
    import torch

    from pipeline_gb300 import datasets
    from pipeline_gb300.batch import BatchOctreeBuilder
    from pipeline_gb300.kernels import k_ComputeMortonCode
    from pipeline_gb300.learned import LearnedCDF
    from pipeline_gb300.pipeline import LearnedOctreeBuilder, OctreeBuilder

    frames, mins, ranges = datasets.scan_frames(256, seed=5)
    fit_f, test_f = frames[:32], frames[32:]
    sizes = [len(f) for f in test_f]
    total = int(sum(sizes))
    stream = torch.cuda.current_stream(dev)
    # model: Morton codes of frames 0-31, each in its own quantisation frame
    codes = []
    for f, mn, rg in zip(fit_f, mins[:32], ranges[:32]):
        p = torch.from_numpy(f).to(dev)
        k = torch.empty(len(f), dtype=torch.int32, device=dev)
        k_ComputeMortonCode(p, k, len(f), mn, rg)
        codes.append(k)
    sample = torch.cat(codes)
    nb = 512
    model = LearnedCDF(max_segments=1024).fit(sample, n_segments=1024, steps=100, lr=0.05,
                                              n_buckets=nb)
    pts = torch.from_numpy(np.concatenate(test_f, 0)).to(dev)
    d_min = torch.tensor(mins[32:], dtype=torch.float32, device=dev)
    d_rg = torch.tensor(ranges[32:], dtype=torch.float32, device=dev)
    b = BatchOctreeBuilder(sizes, device=dev)
    b.capture(pts, d_min, d_rg)
    offs = np.concatenate([[0], np.cumsum(sizes)])
    views = [pts[offs[c]:offs[c + 1]] for c in range(len(sizes))]
    single = OctreeBuilder(max(sizes), device=dev)
    learned = LearnedOctreeBuilder(max(sizes), model, device=dev, n_buckets=nb)

    def plain_loop():
        for v, mn, rg in zip(views, mins[32:], ranges[32:]):
            single.build(v, mn, rg)

    def learned_loop():
        for v, mn, rg in zip(views, mins[32:], ranges[32:]):
            learned.build(v, mn, rg)

    plain_loop()
    learned_loop()
    b.replay()
    torch.cuda.synchronize(dev)
    counts = b.cloud_counts()
    exact, fallbacks, overflow = True, 0, []
    for c in range(0, len(sizes), 16):
        single.build(views[c], mins[32 + c], ranges[32 + c])
        learned.build(views[c], mins[32 + c], ranges[32 + c])
        r, lr_ = single.result(), learned.result()
        st = learned.lsort_stats()
        fallbacks += st["fallback"]
        overflow.append(st["overflow_frac"])
        exact &= r["oct_nodes"].tobytes() == b.cloud_result(c, counts)["oct_nodes"].tobytes()
        exact &= r["oct_nodes"].tobytes() == lr_["oct_nodes"].tobytes()
    # learned + batched: one model (32 buckets per frame) fit on frames 0-31
    # drives the batched build's sort for frames 32-255
    nb_lb = 32
    t0 = time.perf_counter()
    model_lb = LearnedCDF(max_segments=1024).fit(sample, n_segments=1024, steps=100, lr=0.05,
                                                 n_buckets=nb_lb)
    torch.cuda.synchronize(dev)
    fit_lb_ms = (time.perf_counter() - t0) * 1e3
    lbb = BatchOctreeBuilder(sizes, device=dev, model=model_lb, n_buckets=nb_lb)
    lbb.capture(pts, d_min, d_rg)
    lbb.replay()
    torch.cuda.synchronize(dev)
    lb_stats = lbb.learned_stats()
    lb_exact = lbb.same_results(b)
    t_batch = _time_events(b.replay, reps, stream, flush)
    t_lbatch = _time_events(lbb.replay, reps, stream, flush)
    alg = cloud_bytes([(sz, u, bb, m) for sz, (u, bb, m, _) in zip(sizes, counts)])
    t_plain = _time_events(plain_loop, max(2, reps // 4), stream, flush)
    t_learn = _time_events(learned_loop, max(2, reps // 4), stream, flush)
    plain_graph = _graph_of(plain_loop, dev)
    learned_graph = _graph_of(learned_loop, dev)
    t_plain_g = _time_events(plain_graph, max(2, reps // 4), stream, flush) if plain_graph else None
    t_learn_g = _time_events(learned_graph, max(2, reps // 4), stream, flush) if learned_graph else None
    e2e = batches_e2e({"batched": b, "learned_batched": lbb},
                      {"per_frame_plain": single, "per_frame_learned": learned}, pts,
                      np.concatenate(test_f, 0), sizes, mins[32:], ranges[32:], stream, flush,
                      max(2, reps // 4))
    e2e["learned_batched_vs_batched"] = round(e2e["learned_batched_mpts"] / e2e["batched_mpts"], 3)
    return {"workload": "frames: 224 scan-like frames (32-255) of 122,880 points, per-frame "
                        "min/range; model fit on frames 0-31 (1024 segments, 512 buckets)",
            "total_points": total, "batched_mpts": round(total / t_batch / 1e3, 1),
            "per_frame_plain_mpts": round(total / t_plain / 1e3, 1),
            "per_frame_learned_mpts": round(total / t_learn / 1e3, 1),
            "batched_vs_loop": round(t_plain / t_batch, 3),
            "learned_vs_plain_per_frame": round(t_plain / t_learn, 3),
            "per_frame_plain_graph_mpts": round(total / t_plain_g / 1e3, 1) if t_plain_g else None,
            "per_frame_learned_graph_mpts": round(total / t_learn_g / 1e3, 1) if t_learn_g else None,
            "batched_vs_graph_loop": round(t_plain_g / t_batch, 3) if t_plain_g else None,
            "learned_batched_mpts": round(total / t_lbatch / 1e3, 1),
            "hbm_frac_lsd_bytes": {"batched": hbm_frac(alg, t_batch),
                                   "learned_batched": hbm_frac(alg, t_lbatch)},
            "learned_batched_vs_batched": round(t_batch / t_lbatch, 3),
            "learned_batched_vs_graph_loop": round(t_plain_g / t_lbatch, 3) if t_plain_g else None,
            "learned_batched_vs_stream_loop": round(t_plain / t_lbatch, 3),
            "learned_batched_bit_exact_vs_batched": bool(lb_exact),
            "learned_batched_fallback": lb_stats["fallback"],
            "learned_batched_max_bucket": lb_stats["max_bucket"],
            "learned_batched_fit_ms": round(fit_lb_ms, 2),
            "bit_exact_spot_check": bool(exact), "learned_fallbacks_in_spot_check": int(fallbacks),
            "overflow_frac_max": round(max(overflow), 5), "fit_loss": model.header()["loss"],
            "e2e": e2e}


def batches_e2e(batched: dict, single: dict, pts, host_pts, sizes, mins, ranges, stream, flush,
                reps):
    """Batched builds end to end: every cloud's points copied in from pinned
    host memory and its OctNodes copied back (sizes from the node counts read
    back first), either all clouds in one batched build (`batched`: name ->
    captured batch builder) or cloud by cloud through a single-cloud builder
    (`single`: name -> builder), as a per-cloud pipeline does. Mpoints/s over
    the same points and bytes."""
    import torch

    total = int(sum(sizes))
    any_b = next(iter(batched.values()))
    pin_pts = torch.from_numpy(host_pts).pin_memory()
    host_nodes = torch.empty(tuple(any_b.nodes.shape), dtype=any_b.nodes.dtype).pin_memory()
    host_counts = torch.empty(tuple(any_b.counts.shape), dtype=any_b.counts.dtype).pin_memory()
    host_one = torch.empty(4, dtype=torch.int32).pin_memory()
    ns = [int(x) for x in any_b.node_start]
    offs = np.concatenate([[0], np.cumsum(sizes)])
    pin_views = [pin_pts[offs[c]:offs[c + 1]] for c in range(len(sizes))]
    dev_buf = torch.empty((max(sizes), 4), dtype=torch.float32, device=pts.device)
    moved = {"h2d": 0, "d2h": 0}

    def one_batch(builder):
        def step():
            pts.copy_(pin_pts, non_blocking=True)
            builder.replay()
            host_counts.copy_(builder.counts, non_blocking=True)
            stream.synchronize()  # the OctNode counts size the copies
            cnt = host_counts.numpy().reshape(-1, 4)
            d2h = 0
            for c in range(len(sizes)):
                m = int(cnt[c, 2])
                if m:
                    host_nodes[ns[c]:ns[c] + m].copy_(builder.nodes[ns[c]:ns[c] + m],
                                                      non_blocking=True)
                    d2h += m * 60
            moved.update(h2d=pin_pts.numel() * 4, d2h=d2h + host_counts.numel() * 4)
        return step

    def per_cloud(builder):
        def step():
            for c in range(len(sizes)):
                n = int(sizes[c])
                dev_buf[:n].copy_(pin_views[c], non_blocking=True)
                builder.build(dev_buf[:n], float(mins[c]), float(ranges[c]))
                host_one.copy_(builder.d_counts, non_blocking=True)
                stream.synchronize()
                m = int(host_one[2])
                if m:
                    host_nodes[ns[c]:ns[c] + m].copy_(builder.nodes[:m], non_blocking=True)
        return step

    runs = {**{k: one_batch(v) for k, v in batched.items()},
            **{k: per_cloud(v) for k, v in single.items()}}
    t = {}
    for name, fn in runs.items():
        fn()
        torch.cuda.synchronize()
        t[name] = _time_events(fn, reps, stream, flush)
    out = {"mode": "host points in, OctNodes out, each cloud's node count read back first",
           "h2d_bytes": moved["h2d"], "d2h_bytes": moved["d2h"],
           **{f"{k}_mpts": round(total / v / 1e3, 1) for k, v in t.items()}}
    base = next(iter(single))
    for k in batched:
        out[f"{k}_vs_{base}"] = round(t[base] / t[k], 3)
    return out


def sort_bar_workload(dev, flush, reps, pts):
    """The sort stage against CUB's DeviceRadixSort::SortKeys on the same
    16,777,216 Morton codes (30-bit, device-resident, one sort per rep)."""
    import torch

    from pipeline_gb300 import _lib
    from pipeline_gb300.kernels import _workspace, k_ComputeMortonCode

    n = pts.shape[0]
    src = torch.empty(n, dtype=torch.int32, device=dev)
    k_ComputeMortonCode(pts, src, n, MIN_COORD, RANGE)
    keys = torch.empty_like(src)
    alt = torch.empty_like(src)
    stream = torch.cuda.current_stream(dev)
    lib = _lib.load()
    ws = _workspace(lib.oct_sort_workspace_bytes(n, 30), dev)
    sp = C.c_void_p(stream.cuda_stream)

    def ours():
        lib.oct_sort_keys(C.c_void_p(keys.data_ptr()), C.c_void_p(alt.data_ptr()), n, 30,
                          C.c_void_p(ws.data_ptr()), ws.numel(), None, sp)

    def timed(fn):
        ts = []
        for r in range(reps):
            keys.copy_(src)
            flush.fill_(r & 0xFF)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b))
        return statistics.median(ts)

    t_ours = timed(ours)
    ours()
    torch.cuda.synchronize(dev)
    want = torch.sort(src.view(torch.int32))[0]
    ok_ours = torch.equal(keys, want)
    out = {"workload": "sort stage: 16,777,216 30-bit Morton codes of the uniform cloud, "
                       "device-resident", "ours_ms": round(t_ours, 4),
           "ours_gkeys_s": round(n / t_ours / 1e6, 2), "ours_sorted": bool(ok_ours)}
    from cub_bar import build as cub_bar

    path = cub_bar.build()
    if path is None:
        out["cub"] = "unavailable: CUB did not build"
        return out
    bar = C.CDLL(path)
    bar.bar_cub_sort_keys.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                      C.POINTER(C.c_size_t), C.c_void_p]
    tb = C.c_size_t(0)
    bar.bar_cub_sort_keys(None, None, n, 30, None, C.byref(tb), sp)
    temp = torch.empty(max(tb.value, 1), dtype=torch.uint8, device=dev)
    cub_out = torch.empty_like(src)

    def cub():
        bar.bar_cub_sort_keys(C.c_void_p(keys.data_ptr()), C.c_void_p(cub_out.data_ptr()), n, 30,
                              C.c_void_p(temp.data_ptr()), C.byref(tb), sp)

    t_cub = timed(cub)
    out.update({"cub_ms": round(t_cub, 4), "cub_gkeys_s": round(n / t_cub / 1e6, 2),
                "cub_sorted": bool(torch.equal(cub_out, want)),
                "ours_vs_cub": round(t_cub / t_ours, 3)})
    return out


TRAFFIC_FILE = os.path.join(ROOT, "profiles", "dram_traffic_uniform_16m.txt")
TRAFFIC_POINTS = 16777216
TRAFFIC_KERNELS = {"morton+histogram": ["morton_kernel<10, 1>"],
                   "unique": ["unique_count_kernel", "unique_deltas_kernel"],
                   "radix tree+edge count": ["tree_nodes_kernel"],
                   "prefix sum": ["tile_sums_scan_kernel", "edge_scan_kernel"],
                   "octree emit": ["oct_emit_kernel"],
                   "octree finalize": ["oct_finalize_kernel"]}


def read_traffic(kernel_step: str, n: int):
    """DRAM bytes (read + write) of one build step (the sum over its kernels)
    from the committed ncu summary of a 16,777,216-point build (one launch of
    each kernel, measured at that size), scaled by n / 16,777,216 when the
    bench runs another size; None when the summary does not cover every
    kernel of the step."""
    names = TRAFFIC_KERNELS.get(kernel_step)
    if not names or not os.path.exists(TRAFFIC_FILE):
        return None
    found = {}
    with open(TRAFFIC_FILE) as f:
        for ln in f:
            parts = ln.split()
            for name in names:
                if name not in found and len(parts) >= 5 and ln.strip().startswith(name):
                    try:
                        found[name] = float(parts[-4]) + float(parts[-3])
                    except ValueError:
                        pass
    if len(found) != len(names):
        return None
    return int(sum(found.values()) * 1e6 * n / TRAFFIC_POINTS)


def run_sharded_batched(args, rank, world, local_rank):
    """--shard batched: the 512-cloud batch split over the ranks by
    shard_clouds (greedy longest-first on point counts, no collective on the
    data path); each rank builds its clouds in one graph-replayed batched build.
    value = all ranks' points / the slowest rank's time per step."""
    import torch
    import torch.distributed as dist

    from pipeline_gb300 import datasets
    from pipeline_gb300.batch import ShardBuilder

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    clouds = datasets.batched(512, seed=11)
    sizes = [len(c) for c in clouds]
    shard = ShardBuilder(sizes, rank, world, device=dev)
    mine = shard.clouds
    b = shard
    b.capture(clouds, [0.0] * len(sizes), [RANGE] * len(sizes))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    for _ in range(max(args.warmup, 3)):
        b.replay()

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize(dev)

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    barrier()
    for k in range(args.steps):
        flush.fill_(k & 0xFF)
        starts[k].record(stream)
        b.replay()
        ends[k].record(stream)
    barrier()
    ms = statistics.mean(s_.elapsed_time(e_) for s_, e_ in zip(starts, ends))
    if world > 1:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    st = np.array([v[3] for v in b.cloud_counts().values()] or [0], np.int64)
    if int(np.bitwise_or.reduce(st)) != 0:
        raise RuntimeError("device status set")
    total = int(sum(sizes))
    if rank == 0:
        print(json.dumps({
            "metric": "Mpoints/s octree build, batched 512 clouds sharded over ranks",
            "value": round(total / ms / 1e3, 1), "unit": "Mpoints/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
            "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic",
            "config": {"workload": "batched_512 sharded: 512 clouds, sizes log-uniform in [1K, 1M] "
                                   "(seed 11), split over ranks longest-first, no collective",
                       "clouds_rank0": len(mine), "points_rank0": int(sum(sizes[c] for c in mine)),
                       "l2": "flushed between steps (256 MiB write)"}}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the clustered (learned) and batched workloads")
    ap.add_argument("--profile-only", nargs="?", const="plain",
                    choices=["plain", "learned", "clustered", "batched"],
                    help="warm-up builds plus one build, no timing or output (for ncu captures)")
    ap.add_argument("--shard", choices=["batched"], default=None,
                    help="split the 512-cloud batched workload over the ranks (one line)")
    ap.add_argument("--points", type=int, default=N_POINTS,
                    help="cloud size for --profile-only (smaller cases for multi-pass ncu captures)")
    args = ap.parse_args()
    if args.profile_only:
        return profile_only(args)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    try:
        if args.shard == "batched":
            return run_sharded_batched(args, rank, world, local_rank)
        return run_ours(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist

            dist.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
