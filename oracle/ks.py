"""Kuramoto-Sivashinsky state generator (FP64, NumPy) -- oracle / test infrastructure.

This module is part of the CPU oracle.  Only tests, the smoke check and the
CPU-baseline leg of the benchmark use it; the product path never does.

It restates the exponential time-differencing RK4 scheme of Kassam & Trefethen
(SIAM J. Sci. Comput. 26, 2005) as used by the reference generator
``ks_datagen.py:21-101`` for

    u_t = -u u_x - u_xx - u_xxxx,   periodic on [0, L),

with M grid points, real-FFT coefficients in NumPy's unnormalised ``rfft``
convention, 3/2-rule dealiasing of the quadratic term (``ks_datagen.py:57-66``)
and the contour-integral evaluation of the phi-functions with J = 16 points
(``ks_datagen.py:32-48``).

Two initial-condition / warm-up modes exist:

* ``reference_mode``: L = 7*pi, ``uhat[:4] = 0.6``, 10000 warm-up steps
  (``ks_datagen.py:8-25``);
* ``seeded_mode``: L = 22, physical initial state ``0.1 * N(0, 1)`` per grid
  point from ``numpy.random.default_rng(seed)``, the first 1000 time units
  discarded, then one snapshot every ``dt`` -- the synthetic KS workload of the
  benchmarks.
"""
from __future__ import annotations

import numpy as np


class ETDRK4:
    """Precomputed ETDRK4 coefficients for one (L, M, dt)."""

    def __init__(self, L: float, M: int = 64, dt: float = 0.25, J: int = 16):
        self.L, self.M, self.dt = float(L), int(M), float(dt)
        self.M2 = self.M // 2 + 1          # rfft length
        self.Mext = (3 * self.M) // 2      # 3/2-rule padded grid
        k = 2.0 * np.pi / self.L * np.arange(self.M2)
        lin = k ** 2 - k ** 4              # linear operator -d_xx - d_xxxx in Fourier space
        # -1/2 d_x (u^2); the Mext/M factor undoes the scaling of the padded
        # inverse transform (ks_datagen.py:30).
        self.g = -0.5j * (self.Mext / self.M) * k
        self.E = np.exp(dt * lin)
        self.E2 = np.exp(0.5 * dt * lin)
        roots = np.exp(1j * np.pi * (np.arange(1, J + 1) - 0.5) / J)
        z = dt * lin[:, None] + roots[None, :]
        ez = np.exp(z)
        self.Q = dt * np.real(np.mean((np.exp(0.5 * z) - 1.0) / z, axis=1))
        z3 = z ** 3
        self.f1 = dt * np.real(np.mean((-4.0 - z + ez * (4.0 - 3.0 * z + z ** 2)) / z3, axis=1))
        self.f2 = dt * np.real(np.mean(2.0 * (2.0 + z + ez * (-2.0 + z)) / z3, axis=1))
        self.f3 = dt * np.real(np.mean((-4.0 - 3.0 * z - z ** 2 + ez * (4.0 - z)) / z3, axis=1))

    def nonlinear(self, vhat: np.ndarray) -> np.ndarray:
        """Dealiased Fourier coefficients of -u u_x."""
        up = np.fft.irfft(vhat, n=self.Mext)
        return self.g * np.fft.rfft(up ** 2)[: self.M2]

    def step(self, vhat: np.ndarray) -> np.ndarray:
        Nv = self.nonlinear(vhat)
        a = self.E2 * vhat + self.Q * Nv
        Na = self.nonlinear(a)
        b = self.E2 * vhat + self.Q * Na
        Nb = self.nonlinear(b)
        c = self.E2 * a + self.Q * (2.0 * Nb - Nv)
        Nc = self.nonlinear(c)
        return self.E * vhat + self.f1 * Nv + self.f2 * (Na + Nb) + self.f3 * Nc

    def run(self, vhat0: np.ndarray, n_warm: int, n_snap: int) -> np.ndarray:
        """Advance ``n_warm`` steps, then record ``n_snap`` consecutive states
        (the first one is the state after warm-up).  Returns (n_snap, M) float64."""
        v = np.asarray(vhat0, dtype=np.complex128).copy()
        for _ in range(n_warm):
            v = self.step(v)
        out = np.empty((n_snap, self.M), dtype=np.float64)
        if n_snap == 0:
            return out
        out[0] = np.fft.irfft(v, n=self.M)
        for n in range(1, n_snap):
            v = self.step(v)
            out[n] = np.fft.irfft(v, n=self.M)
        return out


def reference_mode(n_snap: int, M: int = 64, n_warm: int = 10000, Lfact: float = 7.0,
                   dt: float = 0.25) -> np.ndarray:
    """States with the reference generator's settings (ks_datagen.py:8-25)."""
    sch = ETDRK4(Lfact * np.pi, M, dt)
    v0 = np.zeros(sch.M2, dtype=np.complex128)
    v0[:4] = 0.6
    return sch.run(v0, n_warm, n_snap)


def seeded_mode(n_snap: int, M: int = 64, L: float = 22.0, seed: int = 0, warm_time: float = 1000.0,
                dt: float = 0.25) -> np.ndarray:
    """Synthetic KS states: random initial state 0.1*N(0,1), warm-up discarded."""
    sch = ETDRK4(L, M, dt)
    u0 = 0.1 * np.random.default_rng(seed).standard_normal(M)
    v0 = np.fft.rfft(u0)
    n_warm = int(round(warm_time / dt))
    return sch.run(v0, n_warm, n_snap)
