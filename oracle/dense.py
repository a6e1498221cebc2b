"""Dense FP64 bistochastic EVD -- oracle / test infrastructure.

Restates ``ks_reference.py:24-40`` with two changes that do not alter the
result: the kernel matrix is built in row blocks (the reference's broadcast
temporary is NM x NM x Nq, ``ks_reference.py:51-57``) and the diagonal
matrices are kept as vectors (``ks_reference.py:26``, ``:29``).

    d = K 1 / NM, q = K d^{-1} / NM,
    Ktilde = D^{-1} K Q^{-1/2}, P = Ktilde Ktilde^T / NM^2,

eigenvalues and eigenvectors returned in descending order
(``ks_reference.py:39-40``).  ``top`` restricts ``eigh`` to the leading
eigenpairs.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla

from .kernel import sqdist_block


def kernel_matrix(X: np.ndarray, scale: float, block: int = 2048) -> np.ndarray:
    X = np.asarray(X, dtype=np.float64)
    N = X.shape[0]
    K = np.empty((N, N), dtype=np.float64)
    for r0 in range(0, N, block):
        K[r0:r0 + block] = np.exp(-scale * sqdist_block(X[r0:r0 + block], X))
    return K


def dense_evd(X: np.ndarray, scale: float, top: int | None = None):
    K = kernel_matrix(X, scale)
    N = K.shape[0]
    d = K.sum(axis=1) / N
    dinv = 1.0 / d
    q = (K @ dinv) / N
    Kt = K * dinv[:, None]
    Kt *= (1.0 / np.sqrt(q))[None, :]
    P = (Kt @ Kt.T) / float(N) ** 2
    del K, Kt
    if top is None:
        w, V = sla.eigh(P)
    else:
        w, V = sla.eigh(P, subset_by_index=[N - top, N - 1])
    return w[::-1].copy(), V[:, ::-1].copy()
