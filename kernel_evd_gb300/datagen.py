"""Synthetic Kuramoto-Sivashinsky states for the workloads (host C stepping).

The phi-function coefficients of the ETDRK4 scheme (Kassam & Trefethen 2005,
contour integral with 16 points, as in ks_datagen.py:32-48) are computed here
with NumPy; the stepping runs in ``libksgen.so`` (csrc/host/ksgen.c).

* ``seeded_states(N, L=22, M=64, seed=0)``: physical initial state
  ``0.1 * N(0, 1)`` per grid point from ``numpy.random.default_rng(seed)``,
  the first ``warm_time`` = 1000 time units discarded, then one state every
  ``dt`` = 0.25 -- the dense d = M workload;
* ``reference_states(n, M=64, Lfact=7)``: the reference generator's settings
  (``uhat[:4] = 0.6``, 10000 warm-up steps), returned as (time, gridpoint).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libksgen.so")
_lib = None


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build with `python -m kernel_evd_gb300.build`")
        lib = C.CDLL(LIB_PATH)
        lib.ks_run.restype = C.c_int
        lib.ks_run.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int64,
                               C.c_void_p, C.c_void_p]
        _lib = lib
    return _lib


def etdrk4_coefficients(L: float, M: int, dt: float, J: int = 16):
    """(coef[6, M2], g[M2]) for E, E2, Q, f1, f2, f3 and the dealiased -1/2 d_x factor."""
    M2 = M // 2 + 1
    Mext = (3 * M) // 2
    k = 2.0 * np.pi / L * np.arange(M2)
    lin = k ** 2 - k ** 4
    g = -0.5j * (Mext / M) * k
    roots = np.exp(1j * np.pi * (np.arange(1, J + 1) - 0.5) / J)
    z = dt * lin[:, None] + roots[None, :]
    ez = np.exp(z)
    z3 = z ** 3
    coef = np.stack([
        np.exp(dt * lin),
        np.exp(0.5 * dt * lin),
        dt * np.real(np.mean((np.exp(0.5 * z) - 1.0) / z, axis=1)),
        dt * np.real(np.mean((-4.0 - z + ez * (4.0 - 3.0 * z + z ** 2)) / z3, axis=1)),
        dt * np.real(np.mean(2.0 * (2.0 + z + ez * (-2.0 + z)) / z3, axis=1)),
        dt * np.real(np.mean((-4.0 - 3.0 * z - z ** 2 + ez * (4.0 - z)) / z3, axis=1)),
    ])
    return np.ascontiguousarray(coef, dtype=np.float64), g.astype(np.complex128)


def run(L: float, M: int, dt: float, vhat0: np.ndarray, n_warm: int, n_snap: int,
        dtype=np.float32) -> np.ndarray:
    coef, g = etdrk4_coefficients(L, M, dt)
    v = np.ascontiguousarray(np.asarray(vhat0, dtype=np.complex128).copy())
    g = np.ascontiguousarray(g)
    out32 = np.empty((n_snap, M), dtype=np.float32) if dtype == np.float32 else None
    out64 = np.empty((n_snap, M), dtype=np.float64) if dtype == np.float64 else None
    st = _load().ks_run(M, coef.ctypes.data, g.ctypes.data, v.ctypes.data, int(n_warm), int(n_snap),
                        out32.ctypes.data if out32 is not None else None,
                        out64.ctypes.data if out64 is not None else None)
    if st != 0:
        raise RuntimeError(f"ks_run failed with status {st}")
    return out32 if out32 is not None else out64


def seeded_states(N: int, L: float = 22.0, M: int = 64, seed: int = 0, warm_time: float = 1000.0,
                  dt: float = 0.25, dtype=np.float32) -> np.ndarray:
    u0 = 0.1 * np.random.default_rng(seed).standard_normal(M)
    return run(L, M, dt, np.fft.rfft(u0), int(round(warm_time / dt)), N, dtype)


def reference_states(n: int, M: int = 64, Lfact: float = 7.0, n_warm: int = 10000, dt: float = 0.25,
                     dtype=np.float32) -> np.ndarray:
    v0 = np.zeros(M // 2 + 1, dtype=np.complex128)
    v0[:4] = 0.6
    return run(Lfact * np.pi, M, dt, v0, n_warm, n, dtype)


# ---- the same trajectories on the GPU (one trajectory per SM) ----------------

def run_gpu(specs, M: int, dt: float = 0.25, n_warm: int = 0, ctx=None, stream=None, precision: str = "fp64"):
    """Advance several trajectories of one grid size M on the GPU
    (``kevd_ks_generate``).  ``specs``: list of (L, vhat0, n_snap); returns a
    list of CUDA float32 tensors (n_snap x M).  The coefficients are the same
    FP64 contour integrals as for the host generator.  ``precision`` "fp64"
    steps like the reference, "fp32" about 20x faster (same attractor, a
    different chaotic trajectory after a few Lyapunov times)."""
    import torch
    from kernel_evd_gb300 import api
    from kernel_evd_gb300._lib import KEVD_FP64, KEVD_MIXED, check
    ctx = ctx or api.Context(0)
    prec = {"fp64": KEVD_FP64, "fp32": KEVD_MIXED}[precision]
    n = len(specs)
    m2 = M // 2 + 1
    coef = np.zeros((n, 6, m2))
    g = np.zeros((n, m2, 2))
    v0 = np.zeros((n, m2, 2))
    outs = []
    for t, (L, vhat0, n_snap) in enumerate(specs):
        c, gg = etdrk4_coefficients(L, M, dt)
        coef[t] = c
        g[t, :, 0], g[t, :, 1] = gg.real, gg.imag
        vv = np.asarray(vhat0, dtype=np.complex128)
        v0[t, :, 0], v0[t, :, 1] = vv.real, vv.imag
        outs.append(torch.empty((int(n_snap), M), dtype=torch.float32, device="cuda"))
    n_snap_arr = np.array([o.shape[0] for o in outs], dtype=np.int64)
    ptrs = (C.c_void_p * n)(*[o.data_ptr() for o in outs])
    st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    check(ctx.lib.kevd_ks_generate(ctx.h, n, M, prec, coef.ctypes.data, g.ctypes.data, v0.ctypes.data, int(n_warm),
                                   n_snap_arr.ctypes.data, ptrs, st), ctx.h)
    return outs


def seeded_states_gpu(N: int, L: float = 22.0, M: int = 64, seed: int = 0, warm_time: float = 1000.0,
                      dt: float = 0.25, ctx=None, precision: str = "fp64"):
    """``seeded_states`` on the GPU (same initial condition, scheme and
    coefficients; FP64 arithmetic in another order, so the chaotic trajectory
    agrees with the host's for a few Lyapunov times and statistically after)."""
    u0 = 0.1 * np.random.default_rng(seed).standard_normal(M)
    return run_gpu([(L, np.fft.rfft(u0), N)], M, dt, int(round(warm_time / dt)), ctx, precision=precision)[0]
