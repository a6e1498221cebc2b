"""Bandwidth calibration (FP64) -- oracle / test infrastructure.

Restates ``ks_bandwidth.cu``:

* pair sums over the strict lower triangle ``T_j = sum_{i>l} exp(-scale_j D_il)``
  (``ks_bandwidth.cu:181-232``, ``:276-325``; the reference additionally divides
  each summand by NM, ``:295``, ``:568-570``);
* the reference's 36-value linear sweep ``1e-3..9e-3, ..., 1..9`` built in
  float32 (``ks_bandwidth.cu:83-91``, ``:419-426``);
* the post-processing on rank 0 (``ks_bandwidth.cu:612-656``):
  ``logS = log(2 T/NM + 1)``, the centred slope, the first arg-max over
  ``i in [0, Nbw-3)``, ``eopt = bw[idmax+1]``, ``mdim = 2 slope[idmax]``;
* the ``bw0.out`` text layout (``ks_bandwidth.cu:645-655``);
* the flat index of the strict lower triangle that the reference's batches walk
  (``tri_count`` / ``tri_ind``, ``ks_bandwidth.cu:104-136``: column-major order, the
  column from a square-root solve in FP64 corrected by integer comparisons), and the
  pair sums taken in that order (``pair_sums_flat``).

It also provides the log-spaced sweep around the median squared distance used
by the dense-state workloads (41 or 64 values in ``2^-10 .. 2^10 x median``).
"""
from __future__ import annotations

import numpy as np

from .kernel import sqdist_block


def reference_sweep() -> np.ndarray:
    """The 36 candidate bandwidths of ks_bandwidth.cu:419-426, float32 as built there."""
    out = []
    for start in (1e-3, 1e-2, 1e-1, 1.0):
        s = np.float32(start)
        for i in range(9):
            out.append(np.float32(s + np.float32(i) * s))
    return np.array(out, dtype=np.float32)


def log_sweep(median: float, n: int, lo: float = -10.0, hi: float = 10.0) -> np.ndarray:
    """n log-spaced eps values in 2^lo .. 2^hi times the median squared distance."""
    return float(median) * 2.0 ** np.linspace(lo, hi, n)


def pair_sums(X: np.ndarray, scales: np.ndarray, block: int = 2048) -> np.ndarray:
    """T_j = sum over i > l of exp(-scales[j] * ||x_i - x_l||^2), FP64."""
    X = np.asarray(X, dtype=np.float64)
    scales = np.asarray(scales, dtype=np.float64)
    N = X.shape[0]
    T = np.zeros(scales.size, dtype=np.float64)
    for r0 in range(0, N, block):
        r1 = min(N, r0 + block)
        D = sqdist_block(X[r0:r1], X[:r1])
        # keep the strict lower triangle: global row i > global column l
        ii = np.arange(r0, r1)[:, None]
        ll = np.arange(r1)[None, :]
        D = D[ii > ll]
        for j, s in enumerate(scales):
            T[j] += np.exp(-s * D).sum()
    return T


def tri_count(k, N: int):
    """Entries of the strict lower triangle of an N x N matrix in the columns before k
    (exact integers)."""
    k = np.asarray(k, dtype=np.int64)
    return k * (2 * N - 1 - k) // 2


def tri_ind(p, N: int):
    """(row, col) of flat indices p of the strict lower triangle, column-major: the
    column is the largest k with tri_count(k) <= p, from the root of the quadratic in
    FP64, truncated, then moved down or up until the integer comparisons hold."""
    p = np.asarray(p, dtype=np.int64)
    a = 2.0 * N - 1.0
    disc = a * a - 8.0 * p.astype(np.float64)
    k = np.trunc((a - np.sqrt(np.maximum(disc, 0.0))) / 2.0).astype(np.int64)
    k = np.maximum(k, 0)
    down = (k > 0) & (tri_count(k, N) > p)
    while down.any():
        k[down] -= 1
        down = (k > 0) & (tri_count(k, N) > p)
    up = tri_count(k + 1, N) <= p
    while up.any():
        k[up] += 1
        up = tri_count(k + 1, N) <= p
    return k + 1 + p - tri_count(k, N), k


def pair_sums_flat(X: np.ndarray, scales: np.ndarray, batch: int = 1 << 16) -> np.ndarray:
    """``pair_sums`` with the pairs visited in batches of the flat index, as the
    reference's distance batches are (``ks_bandwidth.cu:537-577``)."""
    X = np.asarray(X, dtype=np.float64)
    scales = np.asarray(scales, dtype=np.float64)
    N = X.shape[0]
    total = N * (N - 1) // 2
    T = np.zeros(scales.size, dtype=np.float64)
    for p0 in range(0, total, batch):
        i, l = tri_ind(np.arange(p0, min(total, p0 + batch)), N)
        D = ((X[i] - X[l]) ** 2).sum(axis=1)
        for j, s in enumerate(scales):
            T[j] += np.exp(-s * D).sum()
    return T


def select(bw: np.ndarray, T: np.ndarray, NM: int):
    """Post-processing of ks_bandwidth.cu:612-642 in FP64.

    Returns (logS, slope, idmax, eopt, mdim) where slope[i-1] is the centred
    difference at bw[i]."""
    bw = np.asarray(bw, dtype=np.float64)
    T = np.asarray(T, dtype=np.float64)
    nbw = bw.size
    assert nbw >= 3
    logS = np.log(2.0 * T / NM + 1.0)
    logbw = np.log(bw)
    slope = (logS[2:] - logS[:-2]) / (logbw[2:] - logbw[:-2])
    idmax = 0
    for i in range(1, nbw - 2):
        if slope[i] > slope[idmax]:
            idmax = i
    return logS, slope, idmax, float(bw[idmax + 1]), float(2.0 * slope[idmax])


def bw0_text(bw: np.ndarray, logS: np.ndarray, slope: np.ndarray, eopt: float, mdim: float) -> str:
    """bw0.out contents (ks_bandwidth.cu:645-655)."""
    lines = [f"{bw[i]:.5e} {logS[i]:.5e} {slope[i - 1]:.5e}" for i in range(1, len(bw) - 1)]
    return "\n".join(lines) + f"\n\n{eopt:.5e}\n{mdim:.5e}\n"


def median_sqdist_exact(X: np.ndarray, block: int = 2048) -> float:
    """Exact median over all pairs i < l (lower median for an even pair count)."""
    X = np.asarray(X, dtype=np.float64)
    N = X.shape[0]
    parts = []
    for r0 in range(0, N, block):
        r1 = min(N, r0 + block)
        D = sqdist_block(X[r0:r1], X[:r1])
        ii = np.arange(r0, r1)[:, None]
        ll = np.arange(r1)[None, :]
        parts.append(D[ii > ll])
    allD = np.concatenate(parts)
    m = (allD.size - 1) // 2
    return float(np.partition(allD, m)[m])


def sample_pairs(N: int, n_pairs: int, seed: int = 0):
    """Seeded pair sample (i != l) used for the median at large N."""
    rng = np.random.default_rng(seed)
    i = rng.integers(0, N, n_pairs, dtype=np.int64)
    l = rng.integers(0, N - 1, n_pairs, dtype=np.int64)
    l = l + (l >= i)
    return i, l


def median_sqdist_sampled(X: np.ndarray, n_pairs: int = 10_000_000, seed: int = 0) -> float:
    X = np.asarray(X)
    i, l = sample_pairs(X.shape[0], n_pairs, seed)
    D = np.empty(n_pairs, dtype=np.float64)
    for s in range(0, n_pairs, 1 << 20):
        a = np.asarray(X[i[s:s + (1 << 20)]], dtype=np.float64)
        b = np.asarray(X[l[s:s + (1 << 20)]], dtype=np.float64)
        D[s:s + (1 << 20)] = ((a - b) ** 2).sum(axis=1)
    m = (n_pairs - 1) // 2
    return float(np.partition(D, m)[m])
