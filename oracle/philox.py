"""Counter-based uniforms (Philox4x32-10) -- oracle / test infrastructure.

Restates the Philox4x32 block cipher of Salmon, Moraes, Dror & Shaw,
"Parallel random numbers: as easy as 1, 2, 3" (SC'11), ten rounds, and the
uniform mapping the CUDA sampler uses, so that the oracle and the device draw
identical uniforms for a given (seed, round, slot).

Stream layout (shared with ``kernel_evd_gb300/csrc/kevd_rng.cuh``):
counter = (slot, round, stream, 0), key = (seed & 0xffffffff, seed >> 32).
``stream`` 0 feeds the pivot proposals, 1 the accept/reject draws.
The 53-bit uniform is ((w0 >> 5) * 2^26 + (w1 >> 6) + 1) * 2^-53 in (0, 1],
matching the half-open (0, 1] range of the reference's cuRAND draws
(``ks_arpclm.cu:205``, ``:329``).
"""
from __future__ import annotations

import numpy as np

_M0 = np.uint64(0xD2511F53)
_M1 = np.uint64(0xCD9E8D57)
_W0 = np.uint64(0x9E3779B9)
_W1 = np.uint64(0xBB67AE85)
_MASK = np.uint64(0xFFFFFFFF)


def philox4x32(c0, c1, c2, c3, k0, k1, rounds: int = 10):
    """Vectorised Philox4x32; all inputs are uint64 arrays holding 32-bit values."""
    c0, c1, c2, c3 = (np.asarray(v, dtype=np.uint64) & _MASK for v in (c0, c1, c2, c3))
    k0 = np.asarray(k0, dtype=np.uint64) & _MASK
    k1 = np.asarray(k1, dtype=np.uint64) & _MASK
    for _ in range(rounds):
        p0 = _M0 * c0
        p1 = _M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & _MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & _MASK
        c0, c1, c2, c3 = (hi1 ^ c1 ^ k0) & _MASK, lo1, (hi0 ^ c3 ^ k1) & _MASK, lo0
        k0 = (k0 + _W0) & _MASK
        k1 = (k1 + _W1) & _MASK
    return c0, c1, c2, c3


def uniforms(seed: int, rnd: int, stream: int, n: int) -> np.ndarray:
    """n doubles in (0, 1] for slots 0..n-1 of (seed, round, stream)."""
    slot = np.arange(n, dtype=np.uint64)
    z = np.zeros(n, dtype=np.uint64)
    seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    w0, w1, _, _ = philox4x32(slot, z + np.uint64(rnd), z + np.uint64(stream), z,
                              np.uint64(seed & 0xFFFFFFFF), np.uint64(seed >> 32))
    m = (w0 >> np.uint64(5)) * np.uint64(1 << 26) + (w1 >> np.uint64(6))
    return (m.astype(np.float64) + 1.0) * 2.0 ** -53
