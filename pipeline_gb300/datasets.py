"""Seeded synthetic point clouds for the octree-build workloads.

  uniform(n, seed)        n points uniform in [0,1024)^3 through the
                          reference's k_InitRandomVec4 stream (mt19937)
  clustered(n, seed)      mixture of 64 anisotropic Gaussians (per-axis sigma
                          log-uniform in 0.5%..20% of the box, uniform weights,
                          uniform centres) plus 5% uniform noise, clamped to
                          [0, nextafter(1024, 0)] so no coordinate wraps or
                          goes negative
  batched(n_clouds, seed) clouds with sizes log-uniform in [1K, 1M]; even
                          clouds uniform, odd clouds 8-Gaussian mixtures
  scan_frames(n, seed)    lidar-like frames: 64 beams x 1920 azimuth steps,
                          ranges from a ground plane and 40 random boxes with
                          2 cm Gaussian range noise; each frame comes with its
                          own (min_coord, range) so all its points quantise
                          inside the 1024^3 grid

All arrays are float32 [n, 4] with w = 1. Generation runs on the host with
numpy's PCG64 streams; results are deterministic for a seed on one numpy
build (tests compare the GPU against the oracle on the same arrays, so no
cross-machine bit pinning is needed for these generators).
"""
from __future__ import annotations

import numpy as np

BOX = 1024.0
_TOP = np.nextafter(np.float32(BOX), np.float32(0))


def _finish(xyz: np.ndarray) -> np.ndarray:
    out = np.empty((len(xyz), 4), np.float32)
    out[:, :3] = np.clip(xyz, 0.0, _TOP)
    out[:, 3] = 1.0
    return out


def uniform(n: int, seed: int = 114514) -> np.ndarray:
    from .kernels import k_InitRandomVec4

    return k_InitRandomVec4(None, n, 0.0, BOX, seed)


def gaussian_mixture(n: int, k: int, rng: np.random.Generator, noise: float = 0.0,
                     sigma_lo: float = 0.005, sigma_hi: float = 0.20) -> np.ndarray:
    n_noise = int(round(n * noise))
    n_g = n - n_noise
    centres = rng.uniform(0, BOX, (k, 3))
    sig = BOX * np.exp(rng.uniform(np.log(sigma_lo), np.log(sigma_hi), (k, 3)))
    comp = rng.integers(0, k, n_g)
    pts = rng.standard_normal((n_g, 3)) * sig[comp] + centres[comp]
    if n_noise:
        pts = np.concatenate([pts, rng.uniform(0, BOX, (n_noise, 3))], 0)
        pts = pts[rng.permutation(n)]
    return _finish(pts)


def clustered(n: int = 1 << 24, seed: int = 7) -> np.ndarray:
    """64 anisotropic Gaussians + 5% uniform noise (heavy duplicate keys)."""
    rng = np.random.default_rng(seed)
    return gaussian_mixture(n, 64, rng, noise=0.05)


def batched(n_clouds: int = 512, seed: int = 11, lo: int = 1000, hi: int = 1_000_000):
    """List of clouds, sizes log-uniform in [lo, hi]; even uniform, odd 8-Gaussian."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), n_clouds)).astype(np.int64)
    clouds = []
    for c, s in enumerate(sizes):
        if c % 2 == 0:
            clouds.append(_finish(rng.uniform(0, BOX, (int(s), 3))))
        else:
            clouds.append(gaussian_mixture(int(s), 8, rng))
    return clouds


def scan_frames(n_frames: int = 256, seed: int = 5, beams: int = 64, steps: int = 1920):
    """Lidar-like frames. Returns (frames, mins, ranges): frames[f] is
    float32 [beams*steps, 4] in metres; (mins[f], ranges[f]) quantise it."""
    rng = np.random.default_rng(seed)
    elev = np.deg2rad(np.linspace(-24.8, 2.0, beams))
    azim = np.linspace(0, 2 * np.pi, steps, endpoint=False)
    ce, se = np.cos(elev)[:, None], np.sin(elev)[:, None]
    dirs = np.stack([ce * np.cos(azim)[None, :], ce * np.sin(azim)[None, :],
                     np.broadcast_to(se, (beams, steps))], -1).reshape(-1, 3)
    sensor_h = 1.8
    with np.errstate(divide="ignore"):
        inv32 = (1.0 / dirs).astype(np.float32)
    frames, mins, ranges = [], [], []
    for f in range(n_frames):
        # ground plane z = -sensor_h; boxes: centre (x, y), half sizes, height
        boxes = np.stack([rng.uniform(-60, 60, 40), rng.uniform(-60, 60, 40),
                          rng.uniform(0.5, 4, 40), rng.uniform(0.5, 4, 40),
                          rng.uniform(1, 6, 40)], -1)
        t = np.full(len(dirs), 120.0)
        dz = dirs[:, 2]
        ground = np.where(dz < -1e-6, -sensor_h / np.minimum(dz, -1e-6), np.inf)
        t = np.minimum(t, ground)
        # slab test of every ray against every box (float32, axis by axis);
        # the nearest hit wins
        lo = np.stack([boxes[:, 0] - boxes[:, 2], boxes[:, 1] - boxes[:, 3],
                       np.full(len(boxes), -sensor_h)], -1).astype(np.float32)
        hi = np.stack([boxes[:, 0] + boxes[:, 2], boxes[:, 1] + boxes[:, 3],
                       -sensor_h + boxes[:, 4]], -1).astype(np.float32)
        tmin = np.full((len(boxes), len(dirs)), -np.inf, np.float32)
        tmax = np.full((len(boxes), len(dirs)), np.inf, np.float32)
        with np.errstate(divide="ignore", invalid="ignore"):
            for a in range(3):
                t1 = np.multiply.outer(lo[:, a], inv32[:, a])
                t2 = np.multiply.outer(hi[:, a], inv32[:, a])
                np.fmax(tmin, np.fmin(t1, t2), out=tmin)
                np.fmin(tmax, np.fmax(t1, t2), out=tmax)
        hit = (tmax >= np.maximum(tmin, 0)) & (tmin > 0)
        tbox = np.where(hit, tmin, np.float32(np.inf)).min(0)
        t = np.minimum(t, tbox.astype(np.float64))
        t = t + rng.normal(0, 0.02, len(t))
        xyz = (dirs * t[:, None]).astype(np.float32)
        mn = np.float32(xyz.min())
        extent = np.float32(xyz.max() - mn)
        rg = np.float32(extent * (1 + 2.0 ** -20))
        # keep every coordinate strictly below min + range
        while np.any((xyz - mn) / rg * np.float32(1024) >= np.float32(1024)):
            rg = np.nextafter(rg, np.float32(np.inf))
        pts = np.empty((len(xyz), 4), np.float32)
        pts[:, :3] = xyz
        pts[:, 3] = 1
        frames.append(pts)
        mins.append(float(mn))
        ranges.append(float(rg))
    return frames, mins, ranges
