"""Sample views and Gaussian-kernel blocks (FP64) -- oracle / test infrastructure.

Two views of the samples are supported, both reduced to a dense row matrix
``X`` (one sample per row) and a scalar ``scale`` so that

    K(i, j) = exp(-scale * sum_k (X[i,k] - X[j,k])**2).

* Hankel (delay-embedding) view of the reference programs: the input ``u`` has
  ``M`` gridpoints of ``Ndata`` time samples each, time fastest; sample
  ``i`` (gridpoint ``i // N``, time ``i % N``, ``N = Ndata - Nq + 1``) is the
  window ``u[(i//N)*Ndata + i%N : ... + Nq]`` (``ks_arpclm.cu:263-268``,
  ``ks_bandwidth.cu:168-169``), and ``scale = 1 / (Nq * bw)``
  (``ks_arpclm.cu:275``).
* Dense view: ``X`` is an ``N x d`` matrix of states, ``scale = 1 / eps``.

Distances are formed from direct differences, as the reference does
(``ks_arpclm.cu:271-278``, ``ks_reference.py:51-57``), never from a norm
expansion, so the oracle has no cancellation error.
"""
from __future__ import annotations

import numpy as np


def hankel_rows(u: np.ndarray, Ndata: int, M: int, Nq: int) -> np.ndarray:
    """Materialise the delay-embedded samples as an (N*M, Nq) matrix in the
    gridpoint-major order of the CUDA programs (row i -> gridpoint i // N)."""
    u = np.asarray(u)
    N = Ndata - Nq + 1
    assert u.size == Ndata * M
    U = u.reshape(M, Ndata)
    idx = np.arange(N)[:, None] + np.arange(Nq)[None, :]
    return U[:, idx].reshape(M * N, Nq)


def sqdist_block(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    """Squared distances between rows of A (m x d) and B (n x d), FP64, summed
    over the feature index in increasing order."""
    A = np.asarray(A, dtype=np.float64)
    B = np.asarray(B, dtype=np.float64)
    out = np.zeros((A.shape[0], B.shape[0]), dtype=np.float64)
    for k in range(A.shape[1]):
        t = A[:, k][:, None] - B[:, k][None, :]
        out += t * t
    return out


def kblock(X: np.ndarray, rows, cols, scale: float) -> np.ndarray:
    """K(rows, cols) in FP64."""
    X = np.asarray(X)
    A = X[rows] if not isinstance(rows, slice) else X[rows]
    B = X[cols] if not isinstance(cols, slice) else X[cols]
    return np.exp(-scale * sqdist_block(A, B))


def kcols(X: np.ndarray, cols, scale: float, block: int = 65536) -> np.ndarray:
    """K(:, cols) for all rows, blocked over rows."""
    N = X.shape[0]
    cols = np.asarray(cols)
    out = np.empty((N, cols.size), dtype=np.float64)
    B = np.asarray(X[cols], dtype=np.float64)
    for r0 in range(0, N, block):
        out[r0:r0 + block] = np.exp(-scale * sqdist_block(X[r0:r0 + block], B))
    return out
