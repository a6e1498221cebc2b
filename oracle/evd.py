"""Bistochastic normalisation + EVD of a low-rank kernel factor (FP64) -- oracle / test infrastructure.

Restates the closed-form pipeline of ``ks_kevd.cu`` (``README_kevd.md:20-69``).
With ``Khat = F F^T``:

    dtil = Khat 1,  qtil = Khat dtil^{-1},
    P = Dtil^{-1} Khat Qtil^{-1} Khat Dtil^{-1}.

``evd_from_factor`` works on a stored factor ``F``:

    c1 = F^T 1, dtil = F c1, cq = F^T dtil^{-1}, qtil = F cq,
    A = F^T Dtil^{-2} F, s = DBL_EPSILON tr(A), R = chol(A + s I) (upper),
    B = F^T Qtil^{-1} F, W = R B R^T, (lam, V) = eigh(W) ascending,
    Z = R^{-1} V[:, -k_out:], U = Dtil^{-1} F Z.

The trace shift is ``ks_kevd.cu:1447-1499``; the positivity checks and their
abort codes are ``ks_kevd.cu:1170-1181`` (2), ``:1510-1520`` (3),
``:1692-1703`` (4), ``:1904-1913`` (5).  ``evd_from_linv`` follows the
reference's own pass algebra on ``K(:, S)`` and ``L^{-1}`` (``README_kevd.md:40-56``)
and returns its dump intermediates (``ks_kevd.cu:483-484``).
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla

from .kernel import kcols

DBL_EPSILON = np.finfo(np.float64).eps


class EvdError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


def evd_from_factor(F: np.ndarray, k_out: int):
    F = np.asarray(F, dtype=np.float64)
    N, k = F.shape
    c1 = F.sum(axis=0)
    dtil = F @ c1
    if not np.all(dtil > 0):
        raise EvdError(2, "nonpositive dtil")
    dinv = 1.0 / dtil
    cq = F.T @ dinv
    qtil = F @ cq
    if not np.all(qtil > 0):
        raise EvdError(4, "nonpositive qtil")
    Y = F * dinv[:, None]
    A = Y.T @ Y
    trA = float(np.trace(A))
    s = DBL_EPSILON * trA
    try:
        R = sla.cholesky(A + s * np.eye(k), lower=False)
    except np.linalg.LinAlgError as exc:
        raise EvdError(3, "potrf failed") from exc
    Yq = F / np.sqrt(qtil)[:, None]
    B = Yq.T @ Yq
    W = R @ B @ R.T
    W = 0.5 * (W + W.T)
    lam, V = np.linalg.eigh(W)
    Vk = V[:, k - k_out:]
    Z = sla.solve_triangular(R, Vk, lower=False)
    U = (F @ Z) * dinv[:, None]
    return dict(c1=c1, dtil=dtil, cq=cq, qtil=qtil, A=A, trA=trA, shift=s, R=R, B=B, W=W,
                lam=lam, V=V, Z=Z, U=U)


def evd_from_linv(X, scale: float, Linv: np.ndarray, piv: np.ndarray, k_out: int):
    """The reference's four-pass formulation on K(:, S) and L^{-1} (small sizes)."""
    Linv = np.tril(np.asarray(Linv, dtype=np.float64))
    KS = kcols(X, piv, scale)                     # N x r
    c1 = KS.sum(axis=0)                           # pass 1
    p1 = Linv.T @ (Linv @ c1)
    dtil = KS @ p1                                # pass 2
    if not np.all(dtil > 0):
        raise EvdError(2, "nonpositive dtil")
    dinv = 1.0 / dtil
    cq = KS.T @ dinv
    Kt = KS * dinv[:, None]
    Atil = Kt.T @ Kt
    pq = Linv.T @ (Linv @ cq)
    A = Linv @ Atil @ Linv.T                      # dense 1
    trA = float(np.trace(A))
    s = DBL_EPSILON * trA
    R = sla.cholesky(A + s * np.eye(A.shape[0]), lower=False)
    G = R @ Linv
    qtil = KS @ pq                                # pass 3
    if not np.all(qtil > 0):
        raise EvdError(4, "nonpositive qtil")
    Kq = KS / np.sqrt(qtil)[:, None]
    Btil = Kq.T @ Kq
    W = G @ Btil @ G.T                            # dense 2
    W = 0.5 * (W + W.T)
    lam, V = np.linalg.eigh(W)
    r = A.shape[0]
    Vk = V[:, r - k_out:]
    Z = Linv.T @ sla.solve_triangular(R, Vk, lower=False)
    U = (KS @ Z) * dinv[:, None]                  # pass 4
    return dict(c1=c1, p1=p1, dtil=dtil, cq=cq, pq=pq, Atil=Atil, A=A, trA=trA, shift=s, R=R,
                G=G, qtil=qtil, Btil=Btil, W=W, lam=lam, V=V, Z=Z, U=U)


def align_signs(U: np.ndarray, Uref: np.ndarray) -> np.ndarray:
    """Flip columns of U to match the sign of Uref (eigenvectors up to sign)."""
    s = np.sign(np.einsum("ij,ij->j", U, Uref))
    s[s == 0] = 1.0
    return U * s[None, :]


def eigvec_angles(U: np.ndarray, Uref: np.ndarray) -> np.ndarray:
    """Principal angle (radians) between matching columns."""
    U = np.asarray(U, dtype=np.float64)
    Uref = np.asarray(Uref, dtype=np.float64)
    c = np.abs(np.einsum("ij,ij->j", U, Uref))
    c /= np.linalg.norm(U, axis=0) * np.linalg.norm(Uref, axis=0)
    return np.arccos(np.clip(c, -1.0, 1.0))
