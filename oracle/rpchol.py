"""Block randomly pivoted Cholesky with stored factor (FP64) -- oracle / test infrastructure.

Restates the accelerated block RPCholesky of ``ks_arpclm.cu`` (Epperly, Tropp &
Webber; ``README_arpclm.md:21-47``) with the factor ``F`` stored instead of
regenerated.  Per round:

1. propose ``b`` i.i.d. pivots with probability proportional to the residual
   diagonal ``d`` by an inverse-CDF search (``ks_arpclm.cu:197-224``): pivot =
   smallest ``i`` with ``cumsum(d)[i] >= u * sum(d)``, else ``N - 1``;
2. ``H = K(S', S') - F(S', :) F(S', :)^T`` (``ks_arpclm.cu:807-874``; with a
   stored factor the projection term is a row gather of ``F``);
3. sequential accept/reject on ``H`` with ``H0 = diag(H)`` captured first:
   accept proposal ``i`` iff ``H0_i * u_i < H_ii`` and ``H_ii > tol``; on accept
   write the Cholesky column and update the trailing Schur complement
   (``ks_arpclm.cu:305-365``); invert the compacted accepted factor by forward
   substitution (``ks_arpclm.cu:379-394``);
4. new factor columns ``G = (K(:, S_i) - F F(S_i, :)^T) L_i^{-T}`` and
   ``d <- max(d - rowsq(G), 0)`` (``ks_arpclm.cu:933-995``, ``:459-478``);
5. relative trace error ``sum(d) / N`` (``ks_arpclm.cu:538-564``).

``K(:, S) L^{-T} = F`` so this is the same factorisation the reference builds
in its low-memory form; ``linv_from_F`` recovers the reference's ``/linv``
output (``L^{-1}`` with ``L = F(S, :)``) and the pivot list is its ``/spiv``.

Uniforms come from ``philox.uniforms`` (stream 0 = proposals, 1 = accept
draws) or from an injected callable ``draw(round, stream, n)``.
"""
from __future__ import annotations

import numpy as np

from . import philox
from .kernel import kblock, kcols


def propose(d: np.ndarray, u: np.ndarray) -> np.ndarray:
    c = np.cumsum(d)
    p = np.searchsorted(c, u * c[-1], side="left")
    return np.minimum(p, d.size - 1).astype(np.int64)


def reject_and_factor(H: np.ndarray, ua: np.ndarray, tol: float, cap: int):
    """Sequential accept/reject on H (b x b, modified copy); accept at most cap.

    Returns (accpos, Lc, Minv): accepted proposal positions, the compacted
    lower Cholesky factor and its inverse."""
    H = np.array(H, dtype=np.float64, copy=True)
    b = H.shape[0]
    H0 = np.diag(H).copy()
    L = np.zeros((b, b))
    acc = []
    for i in range(b):
        hii = H[i, i]
        if len(acc) < cap and (H0[i] * ua[i] < hii) and (hii > tol):
            acc.append(i)
            L[i:, i] = H[i:, i] / np.sqrt(hii)
            li = L[i + 1:, i]
            H[i + 1:, i + 1:] -= np.outer(li, li)
    acc = np.array(acc, dtype=np.int64)
    Lc = L[np.ix_(acc, acc)]
    n = acc.size
    Minv = np.zeros((n, n))
    if n <= 64:
        # column-wise forward substitution, each sum in increasing e
        for t in range(n):
            Minv[t, t] = 1.0 / Lc[t, t]
            for a in range(t + 1, n):
                s = 0.0
                for e in range(t, a):
                    s += Lc[a, e] * Minv[e, t]
                Minv[a, t] = -s / Lc[a, a]
    else:
        # the same substitution a row at a time (sums in BLAS order: equal to
        # the column-wise form up to rounding; the zeros above the diagonal of
        # Minv add nothing)
        for a in range(n):
            Minv[a, :a] = -(Lc[a, :a] @ Minv[:a, :a]) / Lc[a, a]
            Minv[a, a] = 1.0 / Lc[a, a]
    return acc, Lc, Minv


def rpcholesky(X, scale: float, k_max: int, b: int, tol: float = 1e-10, seed: int = 1234,
               n_rounds: int | None = None, draw=None, err_target: float = 0.0,
               timing: dict | None = None):
    """Stored-factor block RPCholesky.

    Returns dict(F (N x r), piv (r,), err (per round), hm (accepted per round),
    proposals (per round), accpos (per round)).  ``timing``, if given, receives
    the seconds spent in the b x b accept/factor steps (``factor_s``)."""
    X = np.asarray(X)
    N = X.shape[0]
    if draw is None:
        def draw(rnd, stream, n):
            return philox.uniforms(seed, rnd, stream, n)
    if n_rounds is None:
        n_rounds = 1 << 30
    F = np.zeros((N, k_max), dtype=np.float64)
    d = np.ones(N, dtype=np.float64)
    piv = []
    err, hm, props, accs = [], [], [], []
    r = 0
    rnd = 0
    while rnd < n_rounds and r < k_max:
        Sp = propose(d, draw(rnd, 0, b))
        ua = draw(rnd, 1, b)
        Fp = F[Sp, :r]
        H = kblock(X, Sp, Sp, scale) - Fp @ Fp.T
        if timing is not None:
            import time
            t0 = time.perf_counter()
        accpos, Lc, Minv = reject_and_factor(H, ua, tol, k_max - r)
        if timing is not None:
            timing["factor_s"] = timing.get("factor_s", 0.0) + time.perf_counter() - t0
        nacc = accpos.size
        if nacc > 0:
            Si = Sp[accpos]
            G = (kcols(X, Si, scale) - F[:, :r] @ F[Si, :r].T) @ Minv.T
            F[:, r:r + nacc] = G
            d = np.maximum(d - np.einsum("ij,ij->i", G, G), 0.0)
            piv.extend(int(s) for s in Si)
            r += nacc
        err.append(d.sum() / N)
        hm.append(nacc)
        props.append(Sp)
        accs.append(accpos)
        rnd += 1
        if err_target > 0.0 and err[-1] <= err_target:
            break
    return dict(F=F[:, :r], piv=np.array(piv, dtype=np.int64), err=np.array(err),
                hm=np.array(hm, dtype=np.int64), proposals=props, accpos=accs, d=d)


def rpcholesky_linv(X, scale: float, k_max: int, b: int, tol: float = 1e-10, seed: int = 1234,
                    n_rounds: int | None = None, draw=None, rblk: int = 4096):
    """The reference's own round algebra, which never stores F (``ks_arpclm.cu:800-1040``),
    in FP64: ``L^{-1}`` (r x r) and the residual diagonal ``d`` are the whole state.

    * ``P = L^{-1} K(S, S')``, ``H = K(S', S') - P^T P`` (``:807-874``);
    * accept/reject and ``L_i^{-1}`` as in ``reject_and_factor`` (``:877-880``);
    * ``M = L^{-T} L^{-1} K(S, S_i) = L^{-T} P[:, accpos]`` (``:895-927``);
    * per row block R (``rblk`` rows): ``T = K(R, S_i) - K(R, S) M``, ``G = T L_i^{-T}``,
      ``d(R) = max(d(R) - rowsq(G), 0)`` (``:933-995``, ``:459-478``);
    * ``L^{-1}`` grows by the block row ``[-L_i^{-1} M^T | L_i^{-1}]`` (``:489-534``,
      ``:998-1015``).

    Same draws as ``rpcholesky``; returns dict(piv, err, hm, Linv, d)."""
    X = np.asarray(X)
    N = X.shape[0]
    if draw is None:
        def draw(rnd, stream, n):
            return philox.uniforms(seed, rnd, stream, n)
    if n_rounds is None:
        n_rounds = 1 << 30
    Linv = np.zeros((k_max, k_max))
    d = np.ones(N)
    piv = np.zeros(0, dtype=np.int64)
    err, hm = [], []
    rnd = 0
    while rnd < n_rounds and piv.size < k_max:
        r = piv.size
        Sp = propose(d, draw(rnd, 0, b))
        ua = draw(rnd, 1, b)
        P = Linv[:r, :r] @ kblock(X, piv, Sp, scale)
        H = kblock(X, Sp, Sp, scale) - P.T @ P
        accpos, _, Minv = reject_and_factor(H, ua, tol, k_max - r)
        nacc = accpos.size
        if nacc > 0:
            Si = Sp[accpos]
            M = Linv[:r, :r].T @ P[:, accpos]
            for i0 in range(0, N, rblk):
                rows = np.arange(i0, min(N, i0 + rblk))
                T = kblock(X, rows, Si, scale) - kblock(X, rows, piv, scale) @ M
                G = T @ Minv.T
                d[rows] = np.maximum(d[rows] - np.einsum("ij,ij->i", G, G), 0.0)
            Linv[r:r + nacc, :r] = -Minv @ M.T
            Linv[r:r + nacc, r:r + nacc] = np.tril(Minv)
            piv = np.concatenate([piv, Si])
        err.append(d.sum() / N)
        hm.append(nacc)
        rnd += 1
    r = piv.size
    return dict(piv=piv, err=np.array(err), hm=np.array(hm, dtype=np.int64), Linv=Linv[:r, :r], d=d)


def linv_from_F(F: np.ndarray, piv: np.ndarray) -> np.ndarray:
    """L^{-1} with L = F(S, :) lower triangular (the reference's /linv, r x r)."""
    import scipy.linalg as sla
    L = np.tril(np.asarray(F, dtype=np.float64)[piv, :])
    return sla.solve_triangular(L, np.eye(L.shape[0]), lower=True)


def trace_error(X, scale: float, F: np.ndarray, block: int = 65536) -> float:
    """tr(K - F F^T)/tr(K) computed directly (diag(K) = 1)."""
    N = F.shape[0]
    return float((N - np.einsum("ij,ij->", F, F)) / N)
