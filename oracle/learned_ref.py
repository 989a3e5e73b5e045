"""fp64 CPU reference of the learned Morton-key CDF model (test infrastructure).

The GPU fit / inference kernels (pipeline_gb300/csrc/learned.cu) are checked
against this file: loss and gradients within float32 tolerance, bucket ids
exactly (they are integer arithmetic on both sides).

Model. Knots x_0 < x_1 < ... < x_K (x_K = 2^30) are distinct keys taken at
evenly spaced ranks of a sorted training sample. Parameters theta_0..theta_{K-1};
s_m = softplus(theta_m), Z = sum s_m, heights y_k = (sum_{m<k} s_m) / Z, so
y_0 = 0, y_K = 1 and the heights never decrease. For a key v in segment k
(x_k <= v < x_{k+1}; keys below x_0 use segment 0 with f = 0):
    f = (v - x_k) / (x_{k+1} - x_k),   F(v) = y_k + (y_{k+1} - y_k) f.
Training loss on the sorted sample v_0..v_{S-1}: L = mean_i (F(v_i) - (i + 1/2)/S)^2.

Buckets. With NB buckets, fixed-point heights Yq_k = round(y_k NB 2^16)
(made non-decreasing, Yq_0 = 0, Yq_K = NB 2^16) and per-segment slopes
slope_k = floor((Yq_{k+1} - Yq_k) 2^32 / (x_{k+1} - x_k)):
    bucket(v) = min(NB - 1, (Yq_k + ((v - x_k) slope_k >> 32)) >> 16).
(v - x_k) < x_{k+1} - x_k keeps the product below 2^60, so it is exact in
64-bit integers, and bucket(v) never decreases with v — the property that
makes "scatter into buckets, sort each bucket" equal a full sort.
"""
from __future__ import annotations

import numpy as np

KEY_END = 1 << 30
FIX = 16


def knots_from_sorted_sample(sample: np.ndarray, k: int) -> np.ndarray:
    """Distinct knots at evenly spaced ranks of the sorted sample, plus 2^30."""
    s = np.asarray(sample, np.int64)
    idx = (np.arange(k, dtype=np.int64) * len(s)) // k
    x = np.unique(s[idx])
    return np.concatenate([x, [KEY_END]]).astype(np.int64)


def softplus(t):
    return np.where(t > 20, t, np.log1p(np.exp(np.minimum(t, 20))))


def sigmoid(t):
    return 1.0 / (1.0 + np.exp(-t))


def heights(theta: np.ndarray) -> np.ndarray:
    s = softplus(np.asarray(theta, np.float64))
    c = np.concatenate([[0.0], np.cumsum(s)])
    return c / c[-1]


def segments(keys: np.ndarray, x: np.ndarray):
    v = np.asarray(keys, np.int64)
    k = np.searchsorted(x, v, side="right") - 1
    below = k < 0
    k = np.clip(k, 0, len(x) - 2)
    f = (v - x[k]) / (x[k + 1] - x[k]).astype(np.float64)
    f = np.where(below, 0.0, f)
    return k, f


def loss_and_grad(theta: np.ndarray, sorted_sample: np.ndarray, x: np.ndarray):
    theta = np.asarray(theta, np.float64)
    S = len(sorted_sample)
    k, f = segments(sorted_sample, x)
    s = softplus(theta)
    Z = s.sum()
    y = np.concatenate([[0.0], np.cumsum(s)]) / Z
    F = y[k] + (y[k + 1] - y[k]) * f
    t = (np.arange(S) + 0.5) / S
    r = F - t
    L = np.mean(r * r)
    dF = 2.0 * r / S
    K = len(theta)
    g = np.zeros(K + 1)
    np.add.at(g, k, dF * (1.0 - f))
    np.add.at(g, k + 1, dF * f)
    # dL/ds_m = (sum_{k>m} g_k - sum_k g_k y_k) / Z
    suffix = np.cumsum(g[::-1])[::-1]          # suffix[j] = sum_{k>=j} g_k
    gy = np.sum(g * y)
    dL_ds = (suffix[1:] - gy) / Z
    return L, dL_ds * sigmoid(theta)


def fixed_point(theta: np.ndarray, x: np.ndarray, nb: int):
    """(Yq, slope) integer tables for exact bucket assignment."""
    y = heights(theta)
    yq = np.rint(y * (nb << FIX)).astype(np.int64)
    yq = np.maximum.accumulate(yq)
    yq[0] = 0
    yq[-1] = nb << FIX
    yq = np.minimum(yq, nb << FIX)
    w = (x[1:] - x[:-1]).astype(np.int64)
    dy = (yq[1:] - yq[:-1]).astype(object)
    slope = np.array([(int(d) << 32) // int(ww) for d, ww in zip(dy, w)], dtype=np.uint64)
    return yq, slope


def buckets(keys: np.ndarray, x: np.ndarray, yq: np.ndarray, slope: np.ndarray, nb: int) -> np.ndarray:
    v = np.asarray(keys, np.int64)
    k = np.searchsorted(x, v, side="right") - 1
    below = k < 0
    k = np.clip(k, 0, len(x) - 2)
    dv = np.where(below, 0, v - x[k]).astype(np.uint64)
    prod = dv * slope[k]                         # < 2^60: exact in uint64
    fx = yq[k].astype(np.uint64) + (prod >> np.uint64(32))
    b = (fx >> np.uint64(FIX)).astype(np.int64)
    return np.minimum(b, nb - 1)


def adam_fit(sorted_sample, x, steps=200, lr=0.05, theta0=None):
    """Reference training loop (Adam), for tests of the GPU trainer's direction."""
    K = len(x) - 1
    theta = np.full(K, np.log(np.e - 1.0)) if theta0 is None else np.array(theta0, np.float64)
    m = np.zeros(K)
    v = np.zeros(K)
    b1, b2, eps = 0.9, 0.999, 1e-8
    hist = []
    for t in range(1, steps + 1):
        L, g = loss_and_grad(theta, sorted_sample, x)
        hist.append(L)
        m = b1 * m + (1 - b1) * g
        v = b2 * v + (1 - b2) * g * g
        theta -= lr * (m / (1 - b1 ** t)) / (np.sqrt(v / (1 - b2 ** t)) + eps)
    return theta, hist
