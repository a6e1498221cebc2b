"""Out-of-sample (Nystrom) eigenfunctions in FP64 -- oracle / test infrastructure.

The reference's pass 4 (``ks_kevd.cu:2246-2269``) forms, for every training
row ``i``, ``U(i) = dtil(i)^{-1} K(i, S) Z'`` with ``Z' = L^{-T} Z`` and
``dtil(i) = K(i, S) p1``, ``p1 = L^{-T} L^{-1} c``.  With a stored factor
``F = K(:, S) L^{-T}`` (``L = F(S, :)``) that is ``U = Dtil^{-1} F Z``.  The same
formula applied to a new state ``y`` gives its eigenfunction values:

    U(y) = (K(y, S) Z') / (K(y, S) p1'),   Z' = L^{-T} Z,  p1' = L^{-T} c1,

with ``c1 = F^T 1`` and ``Z`` from ``evd_from_factor`` (training rows reproduce
``U`` exactly).
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla

from .evd import evd_from_factor
from .kernel import sqdist_block


def nystrom_model(X: np.ndarray, scale: float, piv: np.ndarray, F: np.ndarray, k_out: int, evd=None):
    """Landmarks ``X[piv]`` and the r x (k_out + 1) matrix ``[Z' | p1']``."""
    piv = np.asarray(piv, dtype=np.int64)
    F = np.asarray(F, dtype=np.float64)[:, :piv.size]
    e = evd if evd is not None else evd_from_factor(F, k_out)
    L = F[piv, :]
    rhs = np.concatenate([e["Z"], e["c1"][:, None]], axis=1)
    zp = sla.solve_triangular(L, rhs, trans="T", lower=True)
    return dict(xs=np.asarray(X, dtype=np.float64)[piv], zp=zp, scale=float(scale), k_out=int(k_out),
                lam=e["lam"])


def nystrom_eval(model, Y: np.ndarray) -> np.ndarray:
    """U(y) for the rows of Y (n x d), FP64."""
    K = np.exp(-model["scale"] * sqdist_block(np.asarray(Y, dtype=np.float64), model["xs"]))
    P = K @ model["zp"]
    return P[:, :-1] / P[:, -1:]
