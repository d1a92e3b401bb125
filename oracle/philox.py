"""Philox4x32-10 counter-based generator and the proposal tape built on it.

TEST INFRASTRUCTURE ONLY: used by tests/, the smoke check and the CPU
baseline to reproduce, on the CPU, the random stream the CUDA sweep draws.

Algorithm: Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as
1, 2, 3", SC'11 (Philox-4x32, 10 rounds), restated from the paper.

Proposal tape.  The reference consumes, per proposal and whatever the
outcome, one draw ``rand(rng, samplers_dict[s_i])`` followed by one
``rand(rng)`` (src/tU/phy_update.jl:259,262; src/tV/phy_update.jl:194,200;
src/tUV/phy_update.jl:192,198).  The sampler picks uniformly among the three
values other than ``s_i`` in ascending order, so a proposal is fully
described by a choice index ``k`` in {0,1,2} and a uniform ``u`` in [0,1).
Proposal ``q`` of sweep ``w`` of chain ``c`` takes one Philox block with
counter (q, w, c, TAPE_STREAM) and key (seed_lo, seed_hi):
    k = (x0 * 3) >> 32
    u = ((x1 >> 5) * 2**26 + (x2 >> 6)) * 2**-53
"""
from __future__ import annotations

import numpy as np

M0, M1 = 0xD2511F53, 0xCD9E8D57
W0, W1 = 0x9E3779B9, 0xBB67AE85
TAPE_STREAM = 0x4B445131
INIT_STREAM = 0x4B445153
MASK = 0xFFFFFFFF


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised Philox4x32-10 over uint64 arrays holding 32-bit words."""
    c0, c1, c2, c3 = (np.asarray(v, dtype=np.uint64) & MASK for v in (c0, c1, c2, c3))
    k0 = np.uint64(k0 & MASK)
    k1 = np.uint64(k1 & MASK)
    m0, m1 = np.uint64(M0), np.uint64(M1)
    for r in range(10):
        if r:
            k0 = (k0 + np.uint64(W0)) & np.uint64(MASK)
            k1 = (k1 + np.uint64(W1)) & np.uint64(MASK)
        p0 = m0 * c0
        p1 = m1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & np.uint64(MASK)
        hi1, lo1 = p1 >> np.uint64(32), p1 & np.uint64(MASK)
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
    return c0, c1, c2, c3


def tape(seed: int, chain: int, sweep: int, n: int):
    """Choice indices ``k`` (uint8) and uniforms ``u`` for proposals 0..n-1."""
    q = np.arange(n, dtype=np.uint64)
    x0, x1, x2, _ = philox4x32_10(q, sweep, chain, TAPE_STREAM, seed & MASK, seed >> 32)
    k = ((x0 * np.uint64(3)) >> np.uint64(32)).astype(np.uint8)
    u = ((x1 >> np.uint64(5)).astype(np.float64) * 67108864.0
         + (x2 >> np.uint64(6)).astype(np.float64)) * (1.0 / 9007199254740992.0)
    return k, u


def initial_field(seed: int, chain: int, n: int) -> np.ndarray:
    """Uniform HS field over {1,2,3,4} for one chain (entry j uses counter j)."""
    j = np.arange(n, dtype=np.uint64)
    x0, _, _, _ = philox4x32_10(j, 0, chain, INIT_STREAM, seed & MASK, seed >> 32)
    return (1 + ((x0 * np.uint64(4)) >> np.uint64(32))).astype(np.uint8)
