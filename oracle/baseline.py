"""Timed CPU form of the pipeline (NumPy / OpenBLAS FP64) -- oracle / test infrastructure.

This is the CPU baseline the benchmark reports beside the GPU numbers: the
reference's CPU path for this pipeline is ``ks_reference.py`` (a dense O(N^3)
EVD, ``ks_reference.py:24-40``), which cannot run at N = 2M; the stored-factor
RPCholesky + bistochastic EVD restated in ``rpchol`` / ``evd`` is the CPU
implementation of the same low-rank pipeline, run here on a row sample.

``timed_pipeline`` separates the work that scales with the number of rows
(kernel columns, residual updates, passes, Grams, U) from the k x k dense
steps (Cholesky, W, eigh, Z), so a time measured on ``n_s`` rows extrapolates
to ``N`` rows as ``stream * N / n_s + dense``.
"""
from __future__ import annotations

import time

import numpy as np
import scipy.linalg as sla

from . import rpchol
from .evd import DBL_EPSILON


def timed_pipeline(X: np.ndarray, scale: float, k: int, b: int, k_out: int, seed: int = 1234):
    t0 = time.perf_counter()
    tm: dict = {}
    r = rpchol.rpcholesky(np.asarray(X, dtype=np.float64), scale, k, b, seed=seed, timing=tm)
    t_rp = time.perf_counter() - t0
    t_fac = tm.get("factor_s", 0.0)
    F = r["F"]
    t1 = time.perf_counter()
    c1 = F.sum(axis=0)
    dtil = F @ c1
    dinv = 1.0 / dtil
    cq = F.T @ dinv
    qtil = F @ cq
    Y = F * dinv[:, None]
    A = Y.T @ Y
    Yq = F / np.sqrt(qtil)[:, None]
    B = Yq.T @ Yq
    t_stream = time.perf_counter() - t1
    t2 = time.perf_counter()
    kk = A.shape[0]
    R = sla.cholesky(A + DBL_EPSILON * np.trace(A) * np.eye(kk), lower=False)
    W = R @ B @ R.T
    W = 0.5 * (W + W.T)
    lam, V = np.linalg.eigh(W)
    Z = sla.solve_triangular(R, V[:, kk - k_out:], lower=False)
    t_dense = time.perf_counter() - t2
    t3 = time.perf_counter()
    U = (F @ Z) * dinv[:, None]
    t_u = time.perf_counter() - t3
    return dict(rpchol_s=t_rp, stream_s=(t_rp - t_fac) + t_stream + t_u, dense_s=t_dense + t_fac,
                lam=lam, U=U,
                trace_error=float(r["err"][-1]), rank=F.shape[1])
